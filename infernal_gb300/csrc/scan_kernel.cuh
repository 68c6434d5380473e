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
// (in shared memory, or in a per-CTA global arena served from L1/L2; see
// scan_plan.h for the layout).  Per state kind:
//   generic states : column-fixed walk, a thread owns one column d and every
//                    rs-th row, four rows of child loads in flight
//   BEGL_S / B     : flattened walk over all cells
//   IL (self-loop on the same row, serial in d) : non-self terms in parallel,
//                    then one thread per row over its band run
//   IR (self-loop on the previous row, serial along a diagonal) : non-self
//                    terms in parallel, then one thread per diagonal
// Each phase's record (descriptor + emission row) arrives by TMA one phase
// ahead, and each phase prefetches the next phase's carry row into registers.
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
#include <cmath>
#include <type_traits>
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
#define CMGB_ATOMIC_OR(p, v) atomicOr((p), (v))
#define CMGB_ATOMIC_MAXU(p, v) atomicMax((p), (v))
#define CMGB_ATOMIC_MINLL(p, v) atomicMin((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXLL(p, v) atomicMax((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXULL(p, v) atomicMax((unsigned long long *) (p), (unsigned long long) (v))
#else
#define CMGB_DEV inline
#define CMGB_SYNC() cmgb_emu_sync()
#define CMGB_LDG(p) (*(p))
#define CMGB_FADD(a, b) ((float) (a) + (float) (b))
#define CMGB_FMUL(a, b) ((float) (a) * (float) (b))
#define CMGB_FDIV(a, b) ((float) (a) / (float) (b))
#define CMGB_I2F(x) ((float) (x))
#define CMGB_ATOMIC_ADD(p, v) __atomic_fetch_add((p), (v), __ATOMIC_SEQ_CST)
#define CMGB_ATOMIC_OR(p, v) __atomic_fetch_or((p), (v), __ATOMIC_SEQ_CST)
#define CMGB_ATOMIC_MAXU(p, v) cmgb_emu_maxu((p), (v))
#define CMGB_ATOMIC_MINLL(p, v) cmgb_emu_minll((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXLL(p, v) cmgb_emu_maxll((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXULL(p, v) cmgb_emu_maxull((unsigned long long *) (p), (unsigned long long) (v))
#endif

#ifndef CMGB_HOST_EMULATION
CMGB_DEV unsigned cmgb_smem_u32(const void *p) { return (unsigned) __cvta_generic_to_shared(p); }
// mbarrier with an arrival count of one (the issuing thread's expect_tx)
CMGB_DEV void cmgb_mbar_init(unsigned long long *mb)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(cmgb_smem_u32(mb)), "r"(1) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// one-dimensional TMA bulk copy global -> shared, completing on mb
CMGB_DEV void cmgb_tma_load(void *dst, const void *src, unsigned bytes, unsigned long long *mb)
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(cmgb_smem_u32(mb)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(cmgb_smem_u32(dst)), "l"(src), "r"(bytes), "r"(cmgb_smem_u32(mb)) : "memory");
}
// bounded wait for phase `parity` of mb; false when the bound is exhausted
CMGB_DEV bool cmgb_mbar_wait(unsigned long long *mb, unsigned parity)
{
  for (int it = 0; it < (1 << 22); it++) {
    unsigned ok;
    asm volatile("{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n selp.b32 %0, 1, 0, P1;\n}"
                 : "=r"(ok) : "r"(cmgb_smem_u32(mb)), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}
CMGB_DEV int __ldg_int(const int *p) { return __ldg(p); }
template <class T> CMGB_DEV T cmgb_shfl_up(T x, int k) { return __shfl_up_sync(0xffffffffu, x, k); }
CMGB_DEV bool cmgb_any(bool b) { return __any_sync(0xffffffffu, b); }
CMGB_DEV void __syncwarp_portable() { __syncwarp(); }
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
  const float *flog;          // FLogsum table (float Inside)
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
  int *err;                   // error word: 1 candidate overflow, 2 a bounded wait ran out
  const unsigned char *rec;   // phase records (descriptor + emission row), see build_records
  float *arena;               // [grid][arena_elems] global tile arena (plans with arena_global)
  // batched scans: window w owns end positions [win_s[w], win_e[w]] and
  // starts computing at win_s0[w] (its sequence's start, or W-1 rows before
  // win_s for a later window of a long sequence); env and best are then
  // per-window arrays
  const long long *win_s, *win_e, *win_s0;
  // multi-model launches: window w belongs to model item_cm[w], whose
  // parameters are multi[item_cm[w]]; cand_tag (the model index) is stored
  // with each candidate cell
  const KParams *multi;
  const int *item_cm;
  int cand_tag;
};

// Order-preserving float <-> uint mapping for atomicMax.
CMGB_DEV unsigned cmgb_f2u(float f)
{
  union { float f; unsigned u; } x; x.f = f;
  return (x.u & 0x80000000u) ? ~x.u : (x.u | 0x80000000u);
}

// Score semirings, selected by ALG: 0 CYK (max, +) over float; 1 integer
// Inside (ILogsum, +) over int (src/logsum.c:87-92); 2 float Inside
// (FLogsum, +) over float (src/logsum.c:160-168).
template <int ALG> struct Sr;
template <> struct Sr<0> {
  typedef float T;
  static CMGB_DEV T imp() { return CMGB_IMP; }
  static CMGB_DEV T add(T a, T b) { return CMGB_FADD(a, b); }
  // ESL_MAX(a,b) = a > b ? a : b.  The max instruction returns the same value
  // and bits except for a = +0, b = -0 (and NaN, which never occurs); a DP value
  // is -0.0 only if a model score table holds -0.0, which log2-odds scores do
  // not (cmgb_model_create checks)
  static CMGB_DEV T comb(T a, T b, const unsigned short *) { return fmaxf(a, b); }
  static CMGB_DEV T rootfirst(T x) { return CMGB_IMP > x ? CMGB_IMP : x; } // ESL_MAX(IMPOSSIBLE, x)
  static CMGB_DEV float score(T x) { return x; }
  static CMGB_DEV float envval(T x) { return x; }
  static CMGB_DEV T init_sc(const StateInfo &s, int d, float el, int) {
    return s.has_end ? CMGB_FADD(CMGB_FMUL(el, CMGB_I2F(d)), s.endsc) : CMGB_IMP;
  }
  // init_sc from hoisted scalars: hasend, endsc (float), iendsc unused
  static CMGB_DEV T init_h(bool hasend, float endsc, int, int d, float el, int) {
    return hasend ? CMGB_FADD(CMGB_FMUL(el, CMGB_I2F(d)), endsc) : CMGB_IMP;
  }
  static CMGB_DEV T init0(const StateInfo &s) { return s.init0; }
  static CMGB_DEV T tsc(const StateInfo &s, int o) { return s.tsc[o]; }
  static CMGB_DEV T beginsc(const StateInfo &s) { return s.beginsc; }
  static CMGB_DEV T esc(const KParams &p, int idx) { return CMGB_LDG(p.oesc + idx); }
  static CMGB_DEV T acc_init() { return -3.0e38f; }
};
template <> struct Sr<1> {
  typedef int T;
  static CMGB_DEV T imp() { return -CMGB_INF; }
  static CMGB_DEV T add(T a, T b) { return a + b; }
  // tbl: the ILogsum table staged in shared memory (entries are 0..1000)
  static CMGB_DEV T comb(T a, T b, const unsigned short *tbl) {
    int mx = a > b ? a : b; mx = mx > -CMGB_INF ? mx : -CMGB_INF;
    int mn = a < b ? a : b;
    // (unsigned) keeps the table index in range even for wrapped int sums,
    // which only arise from residue codes with impossible emission scores
    return (mn <= -CMGB_INF || (unsigned) (mx - mn) >= (unsigned) CMGB_LTBL) ? mx : mx + (int) tbl[mx - mn];
  }
  static CMGB_DEV T rootfirst(T x) { return -CMGB_INF > x ? -CMGB_INF : x; }
  static CMGB_DEV float score(T x) { return x == -CMGB_INF ? CMGB_IMP : CMGB_FDIV(CMGB_I2F(x), 1000.0f); }
  static CMGB_DEV float envval(T x) { return CMGB_I2F(x); }
  static CMGB_DEV T init_sc(const StateInfo &s, int d, float, int iel) {
    return s.has_iend ? iel * d + s.iendsc : -CMGB_INF;
  }
  static CMGB_DEV T init_h(bool hasend, float, int iendsc, int d, float, int iel) {
    return hasend ? iel * d + iendsc : -CMGB_INF;
  }
  static CMGB_DEV T init0(const StateInfo &s) { return s.iinit0; }
  static CMGB_DEV T tsc(const StateInfo &s, int o) { return s.itsc[o]; }
  static CMGB_DEV T beginsc(const StateInfo &s) { return s.ibeginsc; }
  static CMGB_DEV T esc(const KParams &p, int idx) { return CMGB_LDG(p.ioesc + idx); }
  static CMGB_DEV T acc_init() { return (int) 0x80000000; }
};
template <> struct Sr<2> {
  typedef float T;
  static CMGB_DEV T imp() { return CMGB_IMP; }
  static CMGB_DEV T add(T a, T b) { return CMGB_FADD(a, b); }
  // tbl: the FLogsum table (float, in global memory), passed as the same pointer type
  static CMGB_DEV T comb(T a, T b, const unsigned short *tblp) {
    const float *tbl = reinterpret_cast<const float *>(tblp);
    const float mx = a > b ? a : b, mn = a < b ? a : b;
    if (mn == -INFINITY || CMGB_FADD(mx, -mn) >= 23.f) return mx;
    return CMGB_FADD(mx, CMGB_LDG(tbl + (int) CMGB_FMUL(CMGB_FADD(mx, -mn), 1000.0f)));
  }
  static CMGB_DEV T rootfirst(T x) { return CMGB_IMP > x ? CMGB_IMP : x; }
  static CMGB_DEV float score(T x) { return x; }
  static CMGB_DEV float envval(T x) { return x; }
  static CMGB_DEV T init_sc(const StateInfo &s, int d, float el, int) {
    return s.has_end ? CMGB_FADD(CMGB_FMUL(el, CMGB_I2F(d)), s.endsc) : CMGB_IMP;
  }
  static CMGB_DEV T init_h(bool hasend, float endsc, int, int d, float el, int) {
    return hasend ? CMGB_FADD(CMGB_FMUL(el, CMGB_I2F(d)), endsc) : CMGB_IMP;
  }
  static CMGB_DEV T init0(const StateInfo &s) { return s.init0; }
  static CMGB_DEV T tsc(const StateInfo &s, int o) { return s.tsc[o]; }
  static CMGB_DEV T beginsc(const StateInfo &s) { return s.beginsc; }
  static CMGB_DEV T acc_init() { return -3.0e38f; }
};

// Flattened walk over the cells (r, d), r = 1..nrows, d = lo..hi, of one
// phase: thread tid visits cells tid, tid + nt, ... in row-major order with
// an incremental (r, d) update, so the per-cell overhead is a few integer ops.
struct CellWalk {
  int r, d, sr, sdd, hi, wp;
  // wp = hi-lo+1; sr, sdd = nt / wp, nt % wp; inv = 1/wp (host-computed)
  CMGB_DEV CellWalk(int tid, int lo, int hi_, int wp_, int sr_, int sdd_, float inv)
    : sr(sr_), sdd(sdd_), hi(hi_), wp(wp_) {
    int q = (int) ((float) tid * inv);          // tid / wp, corrected below
    if (q * wp > tid) q--;
    if ((q + 1) * wp <= tid) q++;
    r = 1 + q; d = lo + (tid - q * wp);
  }
  CMGB_DEV void next() { d += sdd; r += sr; if (d > hi) { d -= wp; r++; } }
};

// Column-fixed walk over a phase's cells: with wp <= nt columns, thread tid
// owns column tid % wp and rows tid / wp + 1, + rs, ... (rs = nt / wp rows
// per pass; threads past rs * wp idle); wider phases give each thread the
// columns tid, tid + nt, ... and every row.
struct ColWalk { int c0, cstep, r0, rs; };
CMGB_DEV ColWalk col_walk(int wp, int tid, int nt)
{
  ColWalk w;
  if (wp <= nt) {
    w.rs = nt / wp; w.c0 = tid % wp; w.r0 = tid / wp + 1; w.cstep = wp;
    if (w.r0 > w.rs) w.c0 = wp;
  } else { w.rs = 1; w.c0 = tid; w.r0 = 1; w.cstep = nt; }
  return w;
}

// Terms a self-loop chain prefetches ahead of its dependent steps.
#define CMGB_CHUNK 8
// Rows whose child values a generic-cell loop loads before it computes and
// stores any of them (the stores would otherwise hold back the next loads).
#define CMGB_RB 4

// The children terms cv[o] + tv[o] of a non-B cell and its local-end
// term folded in the order of the reference's per-child-count recurrences
// (src/cm_dpsearch.c:307-542); WITH0 adds child 0 last (inserts fold their
// self-loop separately).
template <class R, int CN, bool WITH0, class T>
CMGB_DEV T fold_children(const T (&cv)[CMGB_MAXC], const T (&tv)[CMGB_MAXC], T initv, const unsigned short *tbl)
{
#define CMGB_CH(o) R::add(cv[o], tv[o])
  T sc;
  if (CN == 2) sc = R::comb(CMGB_CH(1), initv, tbl);
  else if (CN == 3) { sc = R::comb(CMGB_CH(2), CMGB_CH(1), tbl); sc = R::comb(sc, initv, tbl); }
  else if (CN == 4) { sc = R::comb(CMGB_CH(3), CMGB_CH(2), tbl); sc = R::comb(sc, initv, tbl); sc = R::comb(sc, CMGB_CH(1), tbl); }
  else if (CN == 5) {
    sc = R::comb(CMGB_CH(4), CMGB_CH(3), tbl); sc = R::comb(sc, initv, tbl); sc = R::comb(sc, CMGB_CH(1), tbl);
    sc = R::comb(sc, CMGB_CH(2), tbl);
  } else {
    sc = R::comb(CMGB_CH(5), initv, tbl); sc = R::comb(sc, CMGB_CH(4), tbl); sc = R::comb(sc, CMGB_CH(3), tbl);
    sc = R::comb(sc, CMGB_CH(2), tbl); sc = R::comb(sc, CMGB_CH(1), tbl);
  }
  if (WITH0) sc = R::comb(sc, CMGB_CH(0), tbl);
#undef CMGB_CH
  return sc;
}

template <int ALG, bool GL, bool MULTI>
CMGB_DEV void qdb_scan_body(const KParams &p0, float *smf, int tid, int nt, int bid)
{
  typedef Sr<ALG> R;
  typedef typename R::T T;
  constexpr bool INS = ALG == 1;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  // the work-queue slot and the two record barriers sit past the plan's arena
  // (a multi-model launch gives every plan the largest smem_elems)
  int *s_win = reinterpret_cast<int *>(smf) + p0.plan.smem_elems;
  unsigned long long *mbar = reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(smf) + p0.plan.smem_elems * 4 + 16);
  // Phase records stream into two shared-memory slots by TMA, one phase
  // ahead: slot g&1 holds the record of the g-th phase this CTA runs.
  unsigned use0 = 0, use1 = 0;   // completed waits per slot (parity source)
  long long g = 0;               // phases run by this CTA
  if (tid == 0) { cmgb_mbar_init(mbar); cmgb_mbar_init(mbar + 1); }

  long long envi = 0x7fffffffffffffffLL, envj = -1;
  float best_root = CMGB_IMP;
  int cur = -1;                  // model whose constants are staged

  for (;;) {
    CMGB_SYNC();
    if (tid == 0) *s_win = CMGB_ATOMIC_ADD(p0.queue, 1);
    CMGB_SYNC();
    const int w = *s_win;
    if (w >= p0.nwin) break;
    const int cm = MULTI ? p0.item_cm[w] : 0;
    const KParams &p = MULTI ? p0.multi[cm] : p0;
    const ScanPlan &P = p.plan;
    const int W = P.W, TT = P.T, NP = P.nphase, Kp = P.Kp;
    // sm: base of the tile buffers, constant row, accumulator and insert scratch
    // (shared memory, or this CTA's slice of the global arena when GL)
    T *sm = GL ? reinterpret_cast<T *>(p.arena) + (size_t) bid * P.arena_elems : reinterpret_cast<T *>(smf);
    T *acc = sm + P.acc_off;
    int *bestr = reinterpret_cast<int *>(sm) + P.bestr_off;
    unsigned char *res = reinterpret_cast<unsigned char *>(smf + P.res_off);
    int *sdesc = reinterpret_cast<int *>(smf) + P.desc_off;
    T *carry0 = reinterpret_cast<T *>(p.carry) + (size_t) bid * 2 * P.carry_elems;
    T *ringb = reinterpret_cast<T *>(p.ring) + (size_t) bid * P.ring_elems;
    const unsigned short *tbl = ALG == 2 ? reinterpret_cast<const unsigned short *>(p.flog)
                                          : reinterpret_cast<const unsigned short *>(smf + P.ltbl_off);
    const float el = P.el_selfsc;
    const int iel = P.iel_selfsc;
    const int accw = P.acc_w, rdn = P.root_dn, rdxW = P.root_dxW, RR = P.ring_rows, tstr = P.tmp_stride;
    const bool want_vsc = p.vsc != nullptr;
    const int slot_words = P.rec_max_bytes / 4;
    if (cm != cur) {
      // this model's constants: the ILogsum table, the constant E row and the
      // record of phase 0 (later windows of the same model find it prefetched
      // by their predecessor's last phase)
      if (INS) {
        unsigned short *t16 = reinterpret_cast<unsigned short *>(smf + P.ltbl_off);
        for (int q = tid; q < CMGB_LTBL; q += nt) t16[q] = (unsigned short) CMGB_LDG(p.ilog + q);
      }
      for (int d = tid; d < P.const_row_len; d += nt) sm[P.const_row + d] = d == 0 ? (T) 0 : R::imp();
      if (tid == 0) {
        const int sl = (int) (g & 1);
        cmgb_tma_load(sdesc + sl * slot_words, p.rec, (unsigned) P.rec0_bytes, mbar + sl);
        if (!cmgb_mbar_wait(mbar + sl, sl ? (use1 & 1) : (use0 & 1))) CMGB_ATOMIC_OR(p.err, 2);
        if (sl) use1++; else use0++;
      }
      CMGB_SYNC();
      cur = cm;
    }
    long long own_s, own_e, s0;
    if (p.win_s) { own_s = p.win_s[w]; own_e = p.win_e[w]; s0 = p.win_s0 ? p.win_s0[w] : own_s; }
    else {
      own_s = p.i0 + (long long) w * p.win_len;
      own_e = own_s + p.win_len - 1;
      if (own_e > p.j0) own_e = p.j0;
      s0 = own_s - (W - 1);
      if (s0 < p.i0) s0 = p.i0;
    }
    const int own_jp = (int) (own_s - s0 + 1);   // first owned row, in window coordinates
    const int last_jp = (int) (own_e - s0 + 1);

    // carry rows of j = s0-1 and the ring row jp = 0 hold the initial matrix values
    for (int k = 0; k < NP; k++) {
      const StateInfo &si = p.st[k];
      if (si.carry >= 0) {
        const T i0v = R::init0(si);
        for (int d = si.lo + tid; d <= si.hi; d += nt) carry0[si.carry + d - si.lo] = d == 0 ? i0v : R::imp();
      }
      if (si.kind == SK_BEGL) {
        const T i0v = R::init0(si);
        for (int d = si.lo + tid; d <= si.hi; d += nt) ringb[si.ring + d - si.lo] = d == 0 ? i0v : R::imp();
      }
    }

    int par = 0;
    for (int jp0 = 0; jp0 < last_jp; jp0 += TT, par ^= 1) {
      const int nrows = (last_jp - jp0) < TT ? (last_jp - jp0) : TT;   // rows jp0+1 .. jp0+nrows
      const T *cin = carry0 + (size_t) par * P.carry_elems;
      T *cout = carry0 + (size_t) (par ^ 1) * P.carry_elems;
      const long long rbase = s0 + jp0 - W;  // res[k] = dsq[rbase + k]; row r's j sits at res[W + r - 1]
      const int ringj = jp0 % RR;            // ring row of jp0
      CMGB_SYNC();
      for (int k = tid; k < P.res_len; k += nt) {
        const long long q = rbase + k;
        unsigned char x = (q >= 0 && q <= p.j0 + 1) ? p.dsq[q] : (unsigned char) 0;
        res[k] = x < Kp ? x : (unsigned char) (Kp - 1);   // codes outside the alphabet read as missing data
      }
      for (int k = tid; k < TT * accw; k += nt) { acc[k] = R::acc_init(); bestr[k] = -1; }
      CMGB_SYNC();
      // carry row of the phase about to run, held in registers (elements tid
      // and tid + nt); each phase loads the next phase's while it works, so
      // no phase starts behind a global-memory read
      T pre0 = R::imp(), pre1 = R::imp();
      {
        const StateInfo &s0i = *reinterpret_cast<const StateInfo *>(sdesc + (int) (g & 1) * slot_words);
        const int c0 = s0i.carry, w0 = s0i.hi - s0i.lo + 1;
        if (c0 >= 0) { if (tid < w0) pre0 = cin[c0 + tid]; if (tid + nt < w0) pre1 = cin[c0 + tid + nt]; }
      }

      for (int k = 0; k < NP; k++, g++) {
        // the record of this phase is in slot g&1 (thread 0 saw its copy
        // complete before the barrier that ended the previous phase)
        const int slot = (int) (g & 1);
        const StateInfo &si = *reinterpret_cast<const StateInfo *>(sdesc + slot * slot_words);
        const T *esc = reinterpret_cast<const T *>(sdesc + slot * slot_words + P.desc_words);
        if (tid == 0) cmgb_tma_load(sdesc + (slot ^ 1) * slot_words, p.rec + si.next_off, (unsigned) si.next_bytes, mbar + (slot ^ 1));
        const T cpre0 = pre0, cpre1 = pre1;
        {
          const int nc = si.next_carry, nw = si.next_cw;
          if (nc >= 0) {
            pre0 = tid < nw ? cin[nc + tid] : R::imp();
            pre1 = tid + nt < nw ? cin[nc + tid + nt] : R::imp();
          }
        }
        // the descriptor fields every phase kind needs, read once into
        // registers (shared-memory stores in the loops would otherwise force
        // re-reads); the branches read their own fields where they start
        const int v = si.v, kind = si.kind, lo = si.lo, hi = si.hi, dn = si.dn, dxW = si.dxW;
        const int cnum = si.cnum, sd = si.sd, emit = si.emit, stride = si.stride, buf = si.buf;
        const int rdo = si.right, has_begin = si.has_begin, carry = si.carry, ringo = si.ring;
        const bool hasend = INS ? (bool) si.has_iend : (bool) si.has_end;
        const float endsc_f = si.endsc;
        const int iendsc_i = si.iendsc;
        const T beg = R::beginsc(si);
        const T imp = R::imp(), i0v = R::init0(si);
        float vbest = CMGB_IMP;
        T tv[CMGB_MAXC];
        int cb[CMGB_MAXC], cs[CMGB_MAXC];
#pragma unroll
        for (int o = 0; o < CMGB_MAXC; o++) { tv[o] = R::tsc(si, o); cb[o] = si.cbuf[o] - si.clo[o]; cs[o] = si.cstr[o]; }
#define INIT(dd) R::init_h(hasend, endsc_f, iendsc_i, (dd), el, iel)
        // row 0 of the state's tile buffer: its last row of the previous tile
#define CMGB_CARRY_IN() do { \
          const int cw_ = hi - lo + 1; \
          if (tid < cw_) sm[buf + tid] = cpre0; \
          if (tid + nt < cw_) sm[buf + tid + nt] = cpre1; \
          for (int x = tid + 2 * nt; x < cw_; x += nt) sm[buf + x] = cin[carry + x]; \
        } while (0)

        if (kind == SK_ROOT) {
          // ---- root: children fold, local-begin accumulator, candidates ----
          const int wpb = si.wp_band, srb = si.sr_band, sddb = si.sdd_band;
          const float invb = si.inv_band;
          for (CellWalk c(tid, dn, dxW, wpb, srb, sddb, invb); c.r <= nrows; c.next()) {
            const int r = c.r, d = c.d, jp = jp0 + r;
            if (d > jp) continue;
            T sc = R::rootfirst(R::add(sm[cb[0] + r * cs[0] + d], tv[0]));
#pragma unroll
            for (int o = 1; o < CMGB_MAXC; o++) if (o < cnum) sc = R::comb(sc, R::add(sm[cb[o] + r * cs[o] + d], tv[o]), tbl);
            const int ai = (r - 1) * accw + d - rdn;
            int br = 0;
            if (!(sc >= acc[ai])) { sc = acc[ai]; br = bestr[ai]; }
            if (jp < own_jp) continue;
            const float f = R::score(sc);
            best_root = best_root > f ? best_root : f;
            const long long j = s0 + jp - 1;
            if (R::envval(sc) >= p.env_cut) {
              const long long ii = j - d + 1;
              envi = envi < ii ? envi : ii;
              envj = envj > j ? envj : j;
            }
            if (d >= 1 && CMGB_NOT_IMP(f) && (p.cand_pos ? (f > 0.0f) : (f >= p.cand_cut))) {
              const int sl = CMGB_ATOMIC_ADD(p.ncand, 1);
              if (sl < p.cand_cap) { Cand cc; cc.j = j; cc.d = d; cc.sc = f; cc.r = br; cc.pad = p.cand_tag; p.cand[sl] = cc; }
              else CMGB_ATOMIC_OR(p.err, 1);
            }
          }
        } else if (kind == SK_IL || kind == SK_IR) {
          // the insert scratch sits in shared memory or, for wide models with a
          // global arena, in the arena; each placement gets its own instance so
          // every access has a known address space (a generic pointer would
          // keep the chains' scratch loads behind their global stores)
          auto insert_phase = [&](T *tmp) {
            // ---- inserts: (1) every term but the self-loop, all band cells in parallel, into tmp ----
            CMGB_CARRY_IN();
  #pragma unroll
            for (int o = 0; o < CMGB_MAXC; o++) cb[o] -= 1;   // children are read at d-1
            if (dn <= dxW) {
              const ColWalk cw = col_walk(dxW - dn + 1, tid, nt);
              auto terms = [&](auto cn_) {
                constexpr int CN = decltype(cn_)::value;
                for (int c = cw.c0; c < dxW - dn + 1; c += cw.cstep) {
                  const int d = dn + c;
                  const T initv = INIT(d - 1);
                  const int rin = d - jp0;       // rows r >= rin hold band cells (d <= jp)
                  int co[CMGB_MAXC];
  #pragma unroll
                  for (int o = 0; o < CMGB_MAXC; o++) co[o] = cb[o] + (cw.r0 - rdo) * cs[o] + d;
                  int to = cw.r0 * tstr + d - lo;
                  int cst[CMGB_MAXC];
#pragma unroll
                  for (int o = 0; o < CMGB_MAXC; o++) cst[o] = cw.rs * cs[o];
                  const int tst = cw.rs * tstr;
                  for (int r = cw.r0; r <= nrows; r += CMGB_RB * cw.rs) {
                    T cv[CMGB_RB][CMGB_MAXC];
#pragma unroll
                    for (int k = 0; k < CMGB_RB; k++) {
                      const bool lv = r + k * cw.rs <= nrows;
#pragma unroll
                      for (int o = 1; o < CMGB_MAXC; o++) if (o < CN) cv[k][o] = lv ? sm[co[o] + k * cst[o]] : imp;
                      cv[k][0] = imp;
                    }
#pragma unroll
                    for (int k = 0; k < CMGB_RB; k++) {
                      const int rk = r + k * cw.rs;
                      if (rk <= nrows && rk >= rin) tmp[to + k * tst] = fold_children<R, CN, false>(cv[k], tv, initv, tbl);
                    }
                    to += CMGB_RB * tst;
#pragma unroll
                    for (int o = 0; o < CMGB_MAXC; o++) co[o] += CMGB_RB * cst[o];
                  }
                }
              };
              switch (cnum) {
                case 2: terms(std::integral_constant<int, 2>()); break;
                case 3: terms(std::integral_constant<int, 3>()); break;
                case 4: terms(std::integral_constant<int, 4>()); break;
                case 5: terms(std::integral_constant<int, 5>()); break;
                default: terms(std::integral_constant<int, 6>()); break;
              }
            }
            CMGB_SYNC();
            // ---- (2) the self-loop chains.  Each row (IL) or diagonal (IR)
            // splits into a pad run, its band run and a pad run, found up front,
            // so a chain step is only its own recurrence; the scratch terms and
            // emission scores are prefetched CMGB_CHUNK steps at a time ----
            const T tself = tv[0];
            if (kind == SK_IR) {
              // IR(r,d) <- IR(r-1,d-1): one thread per diagonal cdg = d - r.  Its
              // cells in [lo, hi] are rows ra..rz; d <= jp holds on a whole
              // diagonal or on none of it (cdg <= jp0), so its band cells are
              // one run b0..b1
              const int ndiag = hi - lo + 1 + TT;
              const int dstep = stride + 1, tstep = tstr + 1;
              const int rvs = own_jp - jp0;
              for (int q = tid; q < ndiag; q += nt) {
                const int cdg = lo - TT + q;
                const int ra = lo - cdg > 1 ? lo - cdg : 1, rz = hi - cdg < nrows ? hi - cdg : nrows;
                if (ra > rz) continue;
                const int b0 = dn - cdg > ra ? dn - cdg : ra;
                const int b1 = cdg > jp0 ? ra - 1 : (dxW - cdg < rz ? dxW - cdg : rz);
                T *out = sm + buf + ra * stride + cdg + ra - lo;
                if (b0 > b1) {   // no band cell on this diagonal
                  for (int r = ra; r <= rz; r++, out += dstep) *out = cdg + r == 0 ? i0v : imp;
                } else {
                  T x = (ra == 1 && cdg >= lo) ? sm[buf + cdg - lo] : imp;   // the diagonal's row-0 cell
                  for (int r = ra; r < b0; r++, out += dstep) { x = cdg + r == 0 ? i0v : imp; *out = x; }
                  for (int r = b0; r <= b1; r += CMGB_CHUNK, out += CMGB_CHUNK * dstep) {
                    const int n = b1 - r + 1;
                    const T *tp = tmp + r * tstr + cdg + r - lo;
                    T tt[CMGB_CHUNK], ee[CMGB_CHUNK];
#pragma unroll
                    for (int u = 0; u < CMGB_CHUNK; u++) {
                      tt[u] = u < n ? tp[u * tstep] : imp;
                      ee[u] = u < n ? esc[res[W + r + u - 1]] : (T) 0;
                    }
#pragma unroll
                    for (int u = 0; u < CMGB_CHUNK; u++) {
                      const T nx = R::add(R::comb(tt[u], R::add(x, tself), tbl), ee[u]);
                      if (u < n) {
                        x = nx;
                        out[u * dstep] = x;
                        if (want_vsc && r + u >= rvs) { const float f = R::score(x); vbest = vbest > f ? vbest : f; }
                      }
                    }
                  }
                  out = sm + buf + (b1 + 1) * stride + cdg + b1 + 1 - lo;
                  for (int r = b1 + 1; r <= rz; r++, out += dstep) *out = cdg + r == 0 ? i0v : imp;
                }
                // the diagonal's row-TT cell is the next tile's carry
                if (TT <= nrows && TT >= ra && TT <= rz) cout[carry + cdg + TT - lo] = sm[buf + TT * stride + cdg + TT - lo];
              }
            } else {
              // IL(r,d) <- IL(r,d-1): one thread per row, serial in d over the band
              for (int r = 1 + tid; r <= nrows; r += nt) {
                const int jp = jp0 + r;
                const int dx = jp < dxW ? jp : dxW;
                T *row = sm + buf + r * stride - lo;
                const T *trow = tmp + r * tstr - lo;
                const bool last = r == TT;
                T *crow = cout + carry - lo;
                const int pad_hi = dn - 1 < hi ? dn - 1 : hi;
                for (int d = lo; d <= pad_hi; d++) { const T pv = d == 0 ? i0v : imp; row[d] = pv; if (last) crow[d] = pv; }
                for (int d = (dx + 1 > dn ? dx + 1 : dn); d <= hi; d++) { const T pv = d == 0 ? i0v : imp; row[d] = pv; if (last) crow[d] = pv; }
                const bool vs = want_vsc && jp >= own_jp;
                T x = (dn - 1 == 0) ? i0v : imp;   // the cell just before the band
                for (int d0 = dn; d0 <= dx; d0 += CMGB_CHUNK) {
                  const int n = dx - d0 + 1;
                  T tt[CMGB_CHUNK], ee[CMGB_CHUNK];
#pragma unroll
                  for (int u = 0; u < CMGB_CHUNK; u++) {
                    tt[u] = u < n ? trow[d0 + u] : imp;
                    ee[u] = u < n ? esc[res[W + r - d0 - u]] : (T) 0;
                  }
#pragma unroll
                  for (int u = 0; u < CMGB_CHUNK; u++) {
                    const T nx = R::add(R::comb(tt[u], R::add(x, tself), tbl), ee[u]);
                    if (u < n) {
                      x = nx;
                      row[d0 + u] = x;
                      if (last) crow[d0 + u] = x;
                      if (vs) { const float f = R::score(x); vbest = vbest > f ? vbest : f; }
                    }
                  }
                }
              }
            }
          };
          if (!GL || P.tmp_smem) insert_phase(reinterpret_cast<T *>(smf) + P.tmp_off);
          else insert_phase(sm + P.tmp_off);
          if (has_begin) {
            CMGB_SYNC();
            for (CellWalk c(tid, dn, dxW, si.wp_band, si.sr_band, si.sdd_band, si.inv_band); c.r <= nrows; c.next()) {
              const int r = c.r, d = c.d, jp = jp0 + r;
              if (d > jp || d < rdn || d > (jp < rdxW ? jp : rdxW)) continue;
              const T cc = R::add(sm[buf + r * stride + d - lo], beg);
              const int ai = (r - 1) * accw + d - rdn;
              if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
            }
          }
        } else {
          // ---- generic, BEGL_S and B: all cells of the phase in parallel ----
          const bool begl = kind == SK_BEGL;
          if (!begl) CMGB_CARRY_IN();
#pragma unroll
          for (int o = 0; o < CMGB_MAXC; o++) cb[o] -= sd;
          if (kind == SK_GEN) {
            // Column-fixed walk: a thread owns one column d of [lo, hi] and
            // every rs-th row, so the band tests, the local-end term and the
            // local-begin test are per column, and each child's address and
            // the emission indices advance by a constant per cell.  The child
            // values (and accumulator cells) of CMGB_RB of the thread's rows
            // are loaded before any of them is computed and stored; rows
            // above the band (d > jp, the window's first rows) are evaluated
            // too (their child reads stay inside the children's buffers) and
            // then take the pad value.
            const ColWalk cw = col_walk(hi - lo + 1, tid, nt);
            auto cells = [&](auto cn_, auto em_) {
              constexpr int CN = decltype(cn_)::value, EM = decltype(em_)::value;
              for (int c = cw.c0; c < hi - lo + 1; c += cw.cstep) {
                const int d = lo + c;
                const T padv = d == 0 ? i0v : imp;
                int oo = buf + cw.r0 * stride + c;
                if (d < dn || d > dxW) {
                  for (int r = cw.r0; r <= nrows; r += cw.rs, oo += cw.rs * stride) {
                    sm[oo] = padv;
                    if (r == TT) cout[carry + c] = padv;
                  }
                  continue;
                }
                const T initv = INIT(d - sd);
                const int rin = d - jp0;       // rows r >= rin hold band cells (d <= jp)
                const int rvs = own_jp - jp0;  // rows r >= rvs are owned by the window
                const bool bcol = has_begin && d >= rdn && d <= rdxW;
                int ao = (cw.r0 - 1) * accw + d - rdn;
                int co[CMGB_MAXC];
#pragma unroll
                for (int o = 0; o < CMGB_MAXC; o++) co[o] = cb[o] + (cw.r0 - rdo) * cs[o] + d;
                int il = W + cw.r0 - d, ir = W + cw.r0 - 1;   // residues i = j-d+1 and j
                int cst[CMGB_MAXC];
#pragma unroll
                for (int o = 0; o < CMGB_MAXC; o++) cst[o] = cw.rs * cs[o];
                const int ost = cw.rs * stride, ast = cw.rs * accw;
                for (int r = cw.r0; r <= nrows; r += CMGB_RB * cw.rs) {
                  T cv[CMGB_RB][CMGB_MAXC], av[CMGB_RB];
#pragma unroll
                  for (int k = 0; k < CMGB_RB; k++) {
                    const bool lv = r + k * cw.rs <= nrows;
#pragma unroll
                    for (int o = 0; o < CMGB_MAXC; o++) if (o < CN) cv[k][o] = lv ? sm[co[o] + k * cst[o]] : imp;
                    av[k] = (lv && bcol) ? acc[ao + k * ast] : imp;
                  }
#pragma unroll
                  for (int k = 0; k < CMGB_RB; k++) {
                    const int rk = r + k * cw.rs;
                    if (rk <= nrows) {
                      T val = fold_children<R, CN, true>(cv[k], tv, initv, tbl);
                      const int ilk = il + k * cw.rs, irk = ir + k * cw.rs;
                      if (EM == 3) val = R::add(val, esc[res[ilk] * Kp + res[irk]]);
                      else if (EM == 1) val = R::add(val, esc[res[ilk]]);
                      else if (EM == 2) val = R::add(val, esc[res[irk]]);
                      if (rk < rin) val = padv;
                      else {
                        if (want_vsc && rk >= rvs) { const float f = R::score(val); vbest = vbest > f ? vbest : f; }
                        if (bcol) {
                          const T cc = R::add(val, beg);
                          if (cc >= av[k]) { acc[ao + k * ast] = cc; bestr[ao + k * ast] = v; }
                        }
                      }
                      sm[oo + k * ost] = val;
                      if (rk == TT) cout[carry + c] = val;
                    }
                  }
                  oo += CMGB_RB * ost; ao += CMGB_RB * ast; il += CMGB_RB * cw.rs; ir += CMGB_RB * cw.rs;
#pragma unroll
                  for (int o = 0; o < CMGB_MAXC; o++) co[o] += CMGB_RB * cst[o];
                }
              }
            };
#define CMGB_EMIT_CASES(CNV) \
            switch (emit) { \
              case 0: cells(std::integral_constant<int, CNV>(), std::integral_constant<int, 0>()); break; \
              case 1: cells(std::integral_constant<int, CNV>(), std::integral_constant<int, 1>()); break; \
              case 2: cells(std::integral_constant<int, CNV>(), std::integral_constant<int, 2>()); break; \
              default: cells(std::integral_constant<int, CNV>(), std::integral_constant<int, 3>()); break; \
            }
            switch (cnum) {
              case 2: CMGB_EMIT_CASES(2) break;
              case 3: CMGB_EMIT_CASES(3) break;
              case 4: CMGB_EMIT_CASES(4) break;
              case 5: CMGB_EMIT_CASES(5) break;
              default: CMGB_EMIT_CASES(6) break;
            }
#undef CMGB_EMIT_CASES
          } else {
          const int banded = si.banded, dn_y = si.dn_y, dx_y = si.dx_y, dn_w = si.dn_w, dx_w = si.dx_w;
          for (CellWalk c(tid, lo, hi, si.wp_all, si.sr_all, si.sdd_all, si.inv_all); c.r <= nrows; c.next()) {
            const int r = c.r, d = c.d, jp = jp0 + r;
            const int dx = jp < dxW ? jp : dxW;
            int rrow = ringj + r; if (rrow >= RR) rrow -= RR;   // ring row of this jp
            T val;
            if (d < dn || d > dx) val = d == 0 ? i0v : imp;
            else {
              if (kind == SK_B) {
                // bifurcation: max/ILogsum over k of BEGL(j-k, d-k) + BEGR(j, k)
                int kmin = 0, kmax = d;
                if (banded) {
                  kmin = dn_y > d - dx_w ? dn_y : d - dx_w; if (kmin < 0) kmin = 0;
                  kmax = dx_y < d - dn_w ? dx_y : d - dn_w;
                }
                val = INIT(d);
                const T *yrow = sm + cb[1] + r * cs[1];
                const T *wring = ringb + cb[0] + d;
                const int wstr = cs[0];
                int rr = rrow - kmin; if (rr < 0) rr += RR;
                int kk = kmin;
                for (; kk + 3 <= kmax; kk += 4) {
                  int r1 = rr - 1; if (r1 < 0) r1 += RR;
                  int r2 = r1 - 1; if (r2 < 0) r2 += RR;
                  int r3 = r2 - 1; if (r3 < 0) r3 += RR;
                  const T a0 = wring[rr * wstr - kk], a1 = wring[r1 * wstr - kk - 1];
                  const T a2 = wring[r2 * wstr - kk - 2], a3 = wring[r3 * wstr - kk - 3];
                  val = R::comb(val, R::add(a0, yrow[kk]), tbl);
                  val = R::comb(val, R::add(a1, yrow[kk + 1]), tbl);
                  val = R::comb(val, R::add(a2, yrow[kk + 2]), tbl);
                  val = R::comb(val, R::add(a3, yrow[kk + 3]), tbl);
                  rr = r3 - 1; if (rr < 0) rr += RR;
                }
                for (; kk <= kmax; kk++) {
                  val = R::comb(val, R::add(wring[rr * wstr - kk], yrow[kk]), tbl);
                  rr = rr == 0 ? RR - 1 : rr - 1;
                }
              } else {   // BEGL_S
                val = INIT(d);
#pragma unroll
                for (int o = 0; o < CMGB_MAXC; o++) if (o < cnum) val = R::comb(val, R::add(sm[cb[o] + r * cs[o] + d], tv[o]), tbl);
              }
              if (want_vsc && jp >= own_jp) { const float f = R::score(val); vbest = vbest > f ? vbest : f; }
              if (has_begin && d >= rdn && d <= (jp < rdxW ? jp : rdxW)) {
                const T cc = R::add(val, beg);
                const int ai = (r - 1) * accw + d - rdn;
                if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
              }
            }
            if (begl) ringb[ringo + rrow * stride + d - lo] = val;
            else {
              sm[buf + r * stride + d - lo] = val;
              if (r == TT) cout[carry + d - lo] = val;
            }
          }
          }
        }
#undef INIT
#undef CMGB_CARRY_IN
        if (want_vsc && vbest > CMGB_IMP) CMGB_ATOMIC_MAXU(p.vsc + v, cmgb_f2u(vbest));
        if (tid == 0) {   // next phase's record, issued at the top of this phase
          const int ns = slot ^ 1;
          if (!cmgb_mbar_wait(mbar + ns, ns ? (use1 & 1) : (use0 & 1))) CMGB_ATOMIC_OR(p.err, 2);
          if (ns) use1++; else use0++;
        }
        CMGB_SYNC();
      }
    }
    if (p.win_s) {   // batched scans: envelope and best score of this sequence
      if (envj >= 0) { CMGB_ATOMIC_MINLL(p.env + 2 * w, envi); CMGB_ATOMIC_MAXLL(p.env + 2 * w + 1, envj); }
      if (best_root > CMGB_IMP) CMGB_ATOMIC_MAXU(p.best + w, cmgb_f2u(best_root));
      envi = 0x7fffffffffffffffLL; envj = -1; best_root = CMGB_IMP;
    }
  }
  // every record copy was waited for by thread 0 before the barrier that followed it
  if (envj >= 0) { CMGB_ATOMIC_MINLL(p0.env, envi); CMGB_ATOMIC_MAXLL(p0.env + 1, envj); }
  if (best_root > CMGB_IMP) CMGB_ATOMIC_MAXU(p0.best, cmgb_f2u(best_root));
}

#ifndef CMGB_HOST_EMULATION
// One 512-thread CTA per SM with up to 128 registers: the generic-cell loops
// keep four rows of child values in flight per thread, which a 64-register
// budget (two CTAs per SM) would spill.
template <int ALG, bool GL, bool MULTI>
__global__ void __launch_bounds__(512, 1) qdb_scan_kernel(KParams p)
{
  extern __shared__ __align__(128) float smem_dyn[];
  qdb_scan_body<ALG, GL, MULTI>(p, smem_dyn, threadIdx.x, blockDim.x, blockIdx.x);
}
#endif
