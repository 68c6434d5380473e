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
#include <cmath>
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
  static CMGB_DEV T comb(T a, T b, const unsigned short *) { return a > b ? a : b; }   // ESL_MAX(a,b)
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
    T *tmp = sm + P.tmp_off;
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

      for (int k = 0; k < NP; k++, g++) {
        // the record of this phase is in slot g&1 (thread 0 saw its copy
        // complete before the barrier that ended the previous phase)
        const int slot = (int) (g & 1);
        const StateInfo &si = *reinterpret_cast<const StateInfo *>(sdesc + slot * slot_words);
        const T *esc = reinterpret_cast<const T *>(sdesc + slot * slot_words + P.desc_words);
        if (tid == 0) cmgb_tma_load(sdesc + (slot ^ 1) * slot_words, p.rec + si.next_off, (unsigned) si.next_bytes, mbar + (slot ^ 1));
        // every descriptor field the phase needs, read once into registers
        // (shared-memory stores in the loops would otherwise force re-reads)
        const int v = si.v, kind = si.kind, lo = si.lo, hi = si.hi, dn = si.dn, dxW = si.dxW;
        const int cnum = si.cnum, sd = si.sd, emit = si.emit, stride = si.stride, buf = si.buf;
        const int rdo = si.right, has_begin = si.has_begin, carry = si.carry, ringo = si.ring;
        const bool hasend = INS ? (bool) si.has_iend : (bool) si.has_end;
        const float endsc_f = si.endsc;
        const int iendsc_i = si.iendsc;
        const int banded = si.banded, dn_y = si.dn_y, dx_y = si.dx_y, dn_w = si.dn_w, dx_w = si.dx_w;
        const int wpa = si.wp_all, sra = si.sr_all, sdda = si.sdd_all, wpb = si.wp_band, srb = si.sr_band, sddb = si.sdd_band;
        const float inva = si.inv_all, invb = si.inv_band;
        const T beg = R::beginsc(si);
        const T imp = R::imp(), i0v = R::init0(si);
        float vbest = CMGB_IMP;
        T tv[CMGB_MAXC];
        int cb[CMGB_MAXC], cs[CMGB_MAXC];
#pragma unroll
        for (int o = 0; o < CMGB_MAXC; o++) { tv[o] = R::tsc(si, o); cb[o] = si.cbuf[o] - si.clo[o]; cs[o] = si.cstr[o]; }
#define INIT(dd) R::init_h(hasend, endsc_f, iendsc_i, (dd), el, iel)

        if (kind == SK_ROOT) {
          // ---- root: children fold, local-begin accumulator, candidates ----
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
          // ---- inserts: (1) every term but the self-loop, all band cells in parallel, into tmp ----
          for (int x = tid; x < hi - lo + 1; x += nt) sm[buf + x] = cin[carry + x];
#pragma unroll
          for (int o = 0; o < CMGB_MAXC; o++) cb[o] -= 1;   // children are read at d-1
          for (CellWalk c(tid, dn, dxW, wpb, srb, sddb, invb); c.r <= nrows; c.next()) {
            const int r = c.r, d = c.d;
            if (d > jp0 + r) continue;
            const int crow = r - rdo;
            T sc;
            switch (cnum) {
#define CH(o) R::add(sm[cb[o] + crow * cs[o] + d], tv[o])
            case 2: sc = R::comb(CH(1), INIT(d - 1), tbl); break;
            case 3: sc = R::comb(CH(2), CH(1), tbl); sc = R::comb(sc, INIT(d - 1), tbl); break;
            case 4: sc = R::comb(CH(3), CH(2), tbl); sc = R::comb(sc, INIT(d - 1), tbl); sc = R::comb(sc, CH(1), tbl); break;
            case 5: sc = R::comb(CH(4), CH(3), tbl); sc = R::comb(sc, INIT(d - 1), tbl); sc = R::comb(sc, CH(1), tbl);
                    sc = R::comb(sc, CH(2), tbl); break;
            default: sc = R::comb(CH(5), INIT(d - 1), tbl); sc = R::comb(sc, CH(4), tbl); sc = R::comb(sc, CH(3), tbl);
                     sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(1), tbl); break;
#undef CH
            }
            tmp[r * tstr + d - lo] = sc;
          }
          CMGB_SYNC();
          // ---- (2) the self-loop chains ----
          const T tself = tv[0];
          if (kind == SK_IR) {
            // IR(r,d) <- IR(r-1,d-1): one thread per diagonal, T short steps
            const T e0 = 0;
            (void) e0;
            const int ndiag = hi - lo + 1 + TT;
            for (int q = tid; q < ndiag; q += nt) {
              const int cdg = lo - TT + q;
              T x = (cdg >= lo && cdg <= hi) ? sm[buf + cdg - lo] : imp;
              for (int r = 1; r <= nrows; r++) {
                const int d = cdg + r;
                if (d < lo || d > hi) { x = imp; continue; }
                const int jp = jp0 + r;
                const int dx = jp < dxW ? jp : dxW;
                T val;
                if (d < dn || d > dx) val = d == 0 ? i0v : imp;
                else {
                  val = R::add(R::comb(tmp[r * tstr + d - lo], R::add(x, tself), tbl), esc[res[W + r - 1]]);
                  if (want_vsc && jp >= own_jp) { const float f = R::score(val); vbest = vbest > f ? vbest : f; }
                }
                sm[buf + r * stride + d - lo] = val;
                if (r == TT) cout[carry + d - lo] = val;
                x = val;
              }
            }
          } else {
            // IL(r,d) <- IL(r,d-1): one warp per row; each lane owns a run of C
            // consecutive cells; carries cross lanes in rounds until no carry
            // changes, which reproduces the sequential chain exactly
            for (int r = 1 + warp; r <= nrows; r += nwarp) {
              const int jp = jp0 + r;
              const int dx = jp < dxW ? jp : dxW;
              T *row = sm + buf + r * stride - lo;
              const T *trow = tmp + r * tstr - lo;
              for (int d = lo + lane; d <= hi; d += 32) if (d < dn || d > dx) row[d] = d == 0 ? i0v : imp;
              const int n = dx - dn + 1;
              if (n > 0) {
                const T start = (dn - 1 == 0) ? i0v : imp;   // the cell just before the band
                const int C = (n + 31) >> 5;
                const int d0 = dn + lane * C;
                const int d1 = (d0 + C - 1 < dx) ? d0 + C - 1 : dx;
                T carry_in = lane == 0 ? start : imp;
                for (int round = 0; round < 33; round++) {
                  T x = carry_in;
                  for (int d = d0; d <= d1; d++) {
                    x = R::add(R::comb(trow[d], R::add(x, tself), tbl), esc[res[W + r - d]]);
                    row[d] = x;
                  }
                  const T out = (d0 <= d1) ? x : carry_in;
                  T nc = cmgb_shfl_up(out, 1);
                  if (lane == 0) nc = start;
                  const bool changed = (d0 <= d1) && (nc != carry_in);
                  carry_in = nc;
                  if (!cmgb_any(changed)) break;
                }
                __syncwarp_portable();
                if (want_vsc && jp >= own_jp)
                  for (int d = dn + lane; d <= dx; d += 32) { const float f = R::score(row[d]); vbest = vbest > f ? vbest : f; }
              }
              __syncwarp_portable();
              if (r == TT) for (int d = lo + lane; d <= hi; d += 32) cout[carry + d - lo] = row[d];
            }
          }
          if (has_begin) {
            CMGB_SYNC();
            for (CellWalk c(tid, dn, dxW, wpb, srb, sddb, invb); c.r <= nrows; c.next()) {
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
          if (!begl) for (int x = tid; x < hi - lo + 1; x += nt) sm[buf + x] = cin[carry + x];
#pragma unroll
          for (int o = 0; o < CMGB_MAXC; o++) cb[o] -= sd;
          if (kind == SK_GEN) {
            // Two cells per iteration: their child loads and folds are
            // independent, so each warp keeps two dependency chains in flight.
            // Both are evaluated at a length clamped into the band (child reads
            // stay inside the children's buffers); pad cells then take their
            // constant value.
            auto gval = [&](int r, int d) -> T {
              const int crow = r - rdo;
              T sc;
#define CH(o) R::add(sm[cb[o] + crow * cs[o] + d], tv[o])
              switch (cnum) {
              case 2: sc = R::comb(CH(1), INIT(d - sd), tbl); sc = R::comb(sc, CH(0), tbl); break;
              case 3: sc = R::comb(CH(2), CH(1), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(0), tbl); break;
              case 4: sc = R::comb(CH(3), CH(2), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(1), tbl);
                      sc = R::comb(sc, CH(0), tbl); break;
              case 5: sc = R::comb(CH(4), CH(3), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(1), tbl);
                      sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(0), tbl); break;
              default: sc = R::comb(CH(5), INIT(d - sd), tbl); sc = R::comb(sc, CH(4), tbl); sc = R::comb(sc, CH(3), tbl);
                       sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(1), tbl); sc = R::comb(sc, CH(0), tbl); break;
              }
#undef CH
              if (emit == 3)      sc = R::add(sc, esc[res[W + r - d] * Kp + res[W + r - 1]]);
              else if (emit == 1) sc = R::add(sc, esc[res[W + r - d]]);
              else if (emit == 2) sc = R::add(sc, esc[res[W + r - 1]]);
              return sc;
            };
            auto finish = [&](int r, int d, T val, bool in) {
              const int jp = jp0 + r;
              if (in) {
                if (want_vsc && jp >= own_jp) { const float f = R::score(val); vbest = vbest > f ? vbest : f; }
                if (has_begin && d >= rdn && d <= (jp < rdxW ? jp : rdxW)) {
                  const T cc = R::add(val, beg);
                  const int ai = (r - 1) * accw + d - rdn;
                  if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
                }
              }
              sm[buf + r * stride + d - lo] = val;
              if (r == TT) cout[carry + d - lo] = val;
            };
            const bool band_ok = dn <= dxW;   // uniform: an empty band has only pad cells
            CellWalk c(tid, lo, hi, wpa, sra, sdda, inva);
            while (c.r <= nrows) {
              CellWalk c2 = c; c2.next();
              const bool two = c2.r <= nrows;
              const int r1 = c.r, d1 = c.d, r2 = two ? c2.r : c.r, d2 = two ? c2.d : c.d;
              const int dx1 = jp0 + r1 < dxW ? jp0 + r1 : dxW, dx2 = jp0 + r2 < dxW ? jp0 + r2 : dxW;
              const bool in1 = d1 >= dn && d1 <= dx1, in2 = d2 >= dn && d2 <= dx2;
              T v1 = d1 == 0 ? i0v : imp, v2 = d2 == 0 ? i0v : imp;
              if (band_ok) {
                const int e1 = d1 < dn ? dn : (d1 > dxW ? dxW : d1), e2 = d2 < dn ? dn : (d2 > dxW ? dxW : d2);
                const T g1 = gval(r1, e1), g2 = gval(r2, e2);
                if (in1) v1 = g1;
                if (in2) v2 = g2;
              }
              finish(r1, d1, v1, in1);
              if (two) finish(r2, d2, v2, in2);
              c = c2;
              if (two) c.next();
            }
          } else
          for (CellWalk c(tid, lo, hi, wpa, sra, sdda, inva); c.r <= nrows; c.next()) {
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
              } else if (begl) {
                val = INIT(d);
#pragma unroll
                for (int o = 0; o < CMGB_MAXC; o++) if (o < cnum) val = R::comb(val, R::add(sm[cb[o] + r * cs[o] + d], tv[o]), tbl);
              } else {
                const int crow = r - rdo;
                T sc;
                switch (cnum) {
#define CH(o) R::add(sm[cb[o] + crow * cs[o] + d], tv[o])
                case 2: sc = R::comb(CH(1), INIT(d - sd), tbl); sc = R::comb(sc, CH(0), tbl); break;
                case 3: sc = R::comb(CH(2), CH(1), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(0), tbl); break;
                case 4: sc = R::comb(CH(3), CH(2), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(1), tbl);
                        sc = R::comb(sc, CH(0), tbl); break;
                case 5: sc = R::comb(CH(4), CH(3), tbl); sc = R::comb(sc, INIT(d - sd), tbl); sc = R::comb(sc, CH(1), tbl);
                        sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(0), tbl); break;
                default: sc = R::comb(CH(5), INIT(d - sd), tbl); sc = R::comb(sc, CH(4), tbl); sc = R::comb(sc, CH(3), tbl);
                         sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(1), tbl); sc = R::comb(sc, CH(0), tbl); break;
#undef CH
                }
                if (emit == 3)      sc = R::add(sc, esc[res[W + r - d] * Kp + res[W + r - 1]]);
                else if (emit == 1) sc = R::add(sc, esc[res[W + r - d]]);
                else if (emit == 2) sc = R::add(sc, esc[res[W + r - 1]]);
                val = sc;
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
#undef INIT
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
// CYK fits 64 registers without spilling, so two 512-thread CTAs (or four of
// 256) share an SM and hide each other's barrier and dependency stalls; the
// Inside kernels keep 128 registers (they spill below that).
template <int ALG, bool GL, bool MULTI>
__global__ void __launch_bounds__(512, (ALG == 0 && !MULTI) ? 2 : 1) qdb_scan_kernel(KParams p)
{
  extern __shared__ __align__(128) float smem_dyn[];
  qdb_scan_body<ALG, GL, MULTI>(p, smem_dyn, threadIdx.x, blockDim.x, blockIdx.x);
}
#endif
