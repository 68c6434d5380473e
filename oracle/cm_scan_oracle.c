/* cm_scan_oracle.c -- CPU restatement of Infernal's QDB scanning DP.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle of the GB300
 * scanners: a plain, row-by-row C statement of the reference algorithms,
 * written for this project from the reference's behaviour.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and only
 * as the checker or the timed CPU baseline; the product library never
 * links, calls or falls back to it.
 *
 * It is pinned against the reference's own scanners compiled from source
 * (oracle/_ref, built by oracle/build_ref.sh) through the golden vectors in
 * tests/golden/, which tests/test_oracle_golden.py replays.
 *
 * Restated functions (reference file:line):
 *   scan_std()            FastCYKScan           src/cm_dpsearch.c:90-681
 *                         FastIInsideScan       src/cm_dpsearch.c:1106-1693
 *                         FastFInsideScan       src/cm_dpsearch.c:1731-2320
 *   band setup            cm_scan_mx_Create     src/cm_mx.c:5725-5738
 *   matrix init           cm_scan_mx_Initialize{Floats,Integers} src/cm_mx.c:6039-6138
 *   init scores           {F,I}CalcInitDPScores src/cm.c:4100-4185
 *   ilogsum()/flogsum()   ILogsum / FLogsum     src/logsum.c:74-92, 138-168
 *   report_greedy()       ReportHitsGreedily    src/cm_mx.c:7547-7628
 *   gamma_update/tback    UpdateGammaHitMx / TBackGammaHitMx src/cm_mx.c:7440-7669
 *   null3_correction()    ScoreCorrectionNull3  src/cm_parsetree.c:2352-2380
 *   core_dinside()        FastFInsideScan's recursion in double with the exact
 *                         log-sum (the FP64 yardstick, not a reference scanner)
 *   remove_overlaps()     cm_tophits_SortForOverlapRemoval + RemoveOrMarkOverlaps
 *                         src/cm_tophits.c:220-245, 400, 1097-1275
 *   oracle_tr_scan()      RefTrCYKScan          src/cm_dpsearch_trunc.c:79-700
 *                         RefITrInsideScan      src/cm_dpsearch_trunc.c:741-1338
 *   tr matrix init        cm_tr_scan_mx_Initialize{Floats,Integers} src/cm_mx.c:6853-6960
 *   fill flags/penalty    cm_TrFillFromPassIdx  src/cm_dpsearch_trunc.c:3566
 *                         cm_tr_penalties_IdxForPass src/cm_trunc.c:464
 *   allow_trunc()         cm_hit_AllowTruncation src/cm_tophits.c:3048-3090
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../include/infernal_gb300.h"

#define IMP      (-1e36f)
#define NOT_IMP(x) ((x) > -9.999e35)
#define INFTY    987654321
#define LOGSUM_TBL 23000
#define MAXC 6
#define MAXF(a, b) (((a) > (b)) ? (a) : (b))
#define MINF(a, b) (((a) < (b)) ? (a) : (b))

enum { ORC_CYK = 0, ORC_IINS = 1, ORC_FINS = 2, ORC_DINS = 3 };

/* ---------------- log-sum tables (src/logsum.c) ---------------- */
static int   ilog_tbl[LOGSUM_TBL];
static float flog_tbl[LOGSUM_TBL];
static int   tables_ready = 0;
static double log2d(double x) { return x > 0 ? log(x) * 1.44269504 : -1e36; }
static void init_tables(void)
{
  if (tables_ready) return;
  for (int i = 0; i < LOGSUM_TBL; i++) {
    ilog_tbl[i] = (int) rint(1000.0f * log2d(1. + exp(((double) -i / 1000.0f) * 0.69314718)));
    flog_tbl[i] = (float) log2d(1. + exp(((double) -i / 1000.0f) * 0.69314718));
  }
  tables_ready = 1;
}
static inline int ilogsum(int a, int b)
{
  int mx = a > b ? a : b; if (mx < -INFTY) mx = -INFTY;
  int mn = a < b ? a : b;
  return (mn <= -INFTY || (mx - mn) >= LOGSUM_TBL) ? mx : mx + ilog_tbl[mx - mn];
}
static inline float flogsum(float a, float b)
{
  float mx = a > b ? a : b, mn = a < b ? a : b;
  return (mn == -INFINITY || (mx - mn) >= 23.f) ? mx : mx + flog_tbl[(int) ((mx - mn) * 1000.0f)];
}
static inline float scorify(int sc) { return sc == -INFTY ? IMP : ((float) sc / 1000.0f); }

/* ---------------- state-type helpers (src/cm.c:1177-1265) ---------------- */
static inline int st_delta(int t)  { return t == CMGB_MP_st ? 2 : (t == CMGB_ML_st || t == CMGB_MR_st || t == CMGB_IL_st || t == CMGB_IR_st) ? 1 : 0; }
static inline int st_right(int t)  { return t == CMGB_MP_st || t == CMGB_MR_st || t == CMGB_IR_st; }
static inline int st_left(int t)   { return t == CMGB_MP_st || t == CMGB_ML_st || t == CMGB_IL_st; }

/* ---------------- hit list ---------------- */
typedef struct { cmgb_hit *h; int64_t n, nalloc; } hitvec;
static void hv_push(hitvec *v, int64_t i, int64_t j, int root, int mode, float sc)
{
  if (v->n == v->nalloc) { v->nalloc = v->nalloc ? 2 * v->nalloc : 64; v->h = realloc(v->h, sizeof(cmgb_hit) * v->nalloc); }
  cmgb_hit *x = &v->h[v->n++];
  x->start = i; x->stop = j; x->root = root; x->mode = mode; x->score = sc;
}

/* ---------------- NULL3 (src/cm_parsetree.c:2352) ---------------- */
static float fsum_kahan(const float *v, int n)
{
  float s = 0.f, c = 0.f, y, t;
  for (int i = 0; i < n; i++) { y = v[i] - c; t = s + y; c = (t - s) - y; s = t; }
  return s;
}
static float null3_correction(const cmgb_model_desc *m, const double *ct_j, const double *ct_im1, int d)
{
  float comp[8];
  int K = m->K;
  for (int a = 0; a < K; a++) comp[a] = (float) (ct_j[a] - ct_im1[a]);
  float s = fsum_kahan(comp, K);
  if (s != 0.f) for (int a = 0; a < K; a++) comp[a] /= s;
  else          for (int a = 0; a < K; a++) comp[a] = 1.f / (float) K;
  float score = 0.;
  for (int a = 0; a < K; a++) score += log2d(comp[a] / m->null[a]) * comp[a] * d;
  score += log2d(m->null3_omega);
  return flogsum(0.f, score);
}

/* residue counts with degenerate codes spread evenly (RNA alphabet) */
static const uint8_t degen_mask[18] = { 1, 2, 4, 8, 0, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 0, 0 };
static void count_residue(double *ct, uint8_t x, int K)
{
  if (x < K) { ct[x] += 1.; return; }
  if (x >= 18) return;
  int n = __builtin_popcount(degen_mask[x]);
  if (n == 0) return;
  for (int y = 0; y < K; y++) if (degen_mask[x] & (1 << y)) ct[y] += 1. / (double) n;
}

/* ---------------- overlap removal (src/cm_tophits.c) ---------------- */
typedef struct { cmgb_hit h; int64_t ord; } ohit;
static int ohit_cmp(const void *a, const void *b)
{
  const ohit *x = a, *y = b;
  if (x->h.score < y->h.score) return 1;
  if (x->h.score > y->h.score) return -1;
  if (x->h.start > y->h.start) return 1;
  if (x->h.start < y->h.start) return -1;
  return (x->ord > y->ord) - (x->ord < y->ord);
}
static void remove_overlaps(hitvec *in, hitvec *out)
{
  int64_t n = in->n;
  ohit *o = malloc(sizeof(ohit) * (n ? n : 1));
  char *rm = calloc(n ? n : 1, 1);
  for (int64_t k = 0; k < n; k++) { o[k].h = in->h[k]; o[k].ord = k; }
  qsort(o, n, sizeof(ohit), ohit_cmp);
  for (int64_t i = 0; i < n; i++) {
    if (rm[i]) continue;
    for (int64_t j = i + 1; j < n; j++)
      if (!rm[j] && !(o[j].h.stop < o[i].h.start) && !(o[i].h.stop < o[j].h.start)) rm[j] = 1;
  }
  for (int64_t i = 0; i < n; i++)
    if (!rm[i]) hv_push(out, o[i].h.start, o[i].h.stop, o[i].h.root, o[i].h.mode, o[i].h.score);
  free(o); free(rm);
}

/* ---------------- the standard scanners ---------------- */
/* Per-scan state shared by the three typed DP cores below. */
typedef struct {
  const cmgb_model_desc *m;
  const uint8_t *dsq;
  int64_t i0, j0, L;
  int M, Wm, W, WP, Kp, K, nbegl;
  const int *dmin, *dmax;
  int *dn, *dxW, *beglidx;
  float cutoff, env_cutoff;
  int want_hits, gamma_mode;
  double (*act)[8];
  float *vsc, vsc_root;
  float *bestf; int *bestr;
  int *bestmode;                 /* truncated scans: mode per d (NULL otherwise) */
  int fill_L, fill_R, fill_T, pass_idx, pty_idx, vmode_root;
  float *gmx; int64_t *gback; float *gsave; int *gr; int *gmode;
  hitvec tmp, fin;
  int64_t envi, envj;
} scanctx;

/* cm_hit_AllowTruncation (src/cm_tophits.c:3048-3090): may a truncated
 * hit of this mode, rooted at state b, be reported in pass pass_idx? */
static int allow_trunc(const cmgb_model_desc *m, int pass_idx, int64_t start, int64_t stop,
                       int64_t i0, int64_t j0, int mode, int b)
{
  const int nd = m->ndidx[b], nt = m->ndtype[nd];
  const int lpos = (nt == CMGB_MATP_nd || nt == CMGB_MATL_nd) ? m->emap_lpos[nd] : m->emap_lpos[nd] + 1;
  const int rpos = (nt == CMGB_MATP_nd || nt == CMGB_MATR_nd) ? m->emap_rpos[nd] : m->emap_rpos[nd] - 1;
  if (pass_idx == CMGB_PASS_STD_ANY || pass_idx == CMGB_PASS_5P_AND_3P_ANY || pass_idx == CMGB_PASS_HMM_ONLY_ANY) return 1;
  if (start == i0 && stop == j0) return 1;
  if (m->flags & CMGB_LOCAL_BEGIN) {
    switch (mode) {
    case CMGB_TRMODE_J: return 1;
    case CMGB_TRMODE_L: return stop == j0;
    case CMGB_TRMODE_R: return start == i0;
    default: return 0;
    }
  }
  switch (mode) {
  case CMGB_TRMODE_J: return lpos == 1 && rpos == m->clen;
  case CMGB_TRMODE_L: return stop == j0 && lpos == 1;
  case CMGB_TRMODE_R: return start == i0 && rpos == m->clen;
  default: return 0;
  }
}

/* per-j hit bookkeeping: ReportHitsGreedily (src/cm_mx.c:7547) or
 * UpdateGammaHitMx (src/cm_mx.c:7440) */
static void report_j(scanctx *c, int64_t j, int64_t jp, int dn0, int dx0)
{
  const int W = c->W;
  if (!c->want_hits) return;
  if (c->gamma_mode) {
    c->gmx[jp] = c->gmx[jp - 1]; c->gback[jp] = -1; c->gsave[jp] = IMP; c->gr[jp] = -1;
    for (int d = MAXF(1, dn0); d <= dx0; d++) {
      int64_t ip = jp - d + 1;
      float hs = c->bestf[d], cum = c->gmx[ip - 1] + hs;
      if (cum > c->gmx[jp] && NOT_IMP(hs)) {
        int rep = 1;
        const int mode = c->bestmode ? c->bestmode[d] : CMGB_TRMODE_J;
        if (c->bestmode) rep = allow_trunc(c->m, c->pass_idx, j - d + 1, j, c->i0, c->j0, mode, c->bestr[d]);
        if (rep && c->act) {
          float c3 = null3_correction(c->m, c->act[jp % (W + 1)], c->act[(ip - 1) % (W + 1)], d);
          hs -= c3; cum -= c3; rep = cum > c->gmx[jp];
        }
        if (rep) { c->gmx[jp] = cum; c->gback[jp] = j - d + 1; c->gsave[jp] = hs; c->gr[jp] = c->bestr[d]; c->gmode[jp] = mode; }
      }
    }
  } else {
    float best = IMP;
    for (int d = MAXF(1, dn0); d <= dx0; d++) {
      float hs = c->bestf[d];
      if (hs > best && hs >= c->cutoff && NOT_IMP(hs)) {
        int rep = 1;
        const int mode = c->bestmode ? c->bestmode[d] : CMGB_TRMODE_J;
        if (c->bestmode) rep = allow_trunc(c->m, c->pass_idx, j - d + 1, j, c->i0, c->j0, mode, c->bestr[d]);
        if (rep && c->act) {
          int64_t ip = jp - d + 1;
          hs -= null3_correction(c->m, c->act[jp % (W + 1)], c->act[(ip - 1) % (W + 1)], d);
          rep = (hs > best && hs >= c->cutoff);
        }
        if (rep) { hv_push(&c->tmp, j - d + 1, j, c->bestr[d], mode, hs); best = hs; }
      }
    }
  }
}

/* The typed DP core is written once in cm_scan_oracle_core.h and instantiated
 * for CYK (float max), integer Inside (ILogsum) and float Inside (FLogsum). */
#define CORE_NAME core_cyk
#define SCT float
#define IMPV IMP
#define COMB(a, b) MAXF((a), (b))
#define ROOTFIRST(x) MAXF(IMP, (x))
#define SCOREF(x) (x)
#define ENVF(x) (x)
#define TSC(v, o) m->tsc[(v) * MAXC + (o)]
#define ESC(v) (m->oesc + (size_t) (v) * Kp * Kp)
#define ESCT float
#define EV(x) (x)
#define BEGINSC(y) m->beginsc[y]
#define HAS_BEGIN(y) NOT_IMP(m->beginsc[y])
#define ENDSC(v) m->endsc[v]
#define INIT_SC(v, d) (NOT_IMP(m->endsc[v]) ? (float) (m->el_selfsc * (d)) + m->endsc[v] : IMP)
#include "cm_scan_oracle_core.h"

#define CORE_NAME core_finside
#define SCT float
#define IMPV IMP
#define COMB(a, b) flogsum((a), (b))
#define ROOTFIRST(x) MAXF(IMP, (x))
#define SCOREF(x) (x)
#define ENVF(x) (x)
#define TSC(v, o) m->tsc[(v) * MAXC + (o)]
#define ESC(v) (m->oesc + (size_t) (v) * Kp * Kp)
#define ESCT float
#define EV(x) (x)
#define BEGINSC(y) m->beginsc[y]
#define HAS_BEGIN(y) NOT_IMP(m->beginsc[y])
#define ENDSC(v) m->endsc[v]
#define INIT_SC(v, d) (NOT_IMP(m->endsc[v]) ? (float) (m->el_selfsc * (d)) + m->endsc[v] : IMP)
#include "cm_scan_oracle_core.h"

#define CORE_NAME core_iinside
#define SCT int
#define IMPV (-INFTY)
#define COMB(a, b) ilogsum((a), (b))
#define ROOTFIRST(x) (((x) > -INFTY) ? (x) : -INFTY)
#define SCOREF(x) scorify(x)
#define ENVF(x) ((float) (x))
#define TSC(v, o) m->itsc[(v) * MAXC + (o)]
#define ESC(v) (m->ioesc + (size_t) (v) * Kp * Kp)
#define ESCT int
#define EV(x) (x)
#define BEGINSC(y) m->ibeginsc[y]
#define HAS_BEGIN(y) (m->ibeginsc[y] != -INFTY)
#define ENDSC(v) m->iendsc[v]
#define INIT_SC(v, d) ((m->iendsc[v] != -INFTY) ? m->iel_selfsc * (d) + m->iendsc[v] : -INFTY)
#include "cm_scan_oracle_core.h"

/* Double-precision Inside: the FastFInsideScan recursion in double with the
 * exact log2(2^a + 2^b) instead of the FLogsum table, and IMPOSSIBLE scores
 * mapped to -infinity.  Not a reference scanner: the yardstick for the
 * table-based Inside scores. */
static inline double dlogsum(double a, double b)
{
  const double mx = a > b ? a : b, mn = a < b ? a : b;
  if (mn == -INFINITY) return mx;
  return mx + log2(1.0 + exp2(mn - mx));
}
static inline double dsc(float x) { return NOT_IMP(x) ? (double) x : -INFINITY; }
#define CORE_NAME core_dinside
#define SCT double
#define IMPV (-INFINITY)
#define COMB(a, b) dlogsum((a), (b))
#define ROOTFIRST(x) (x)
#define SCOREF(x) ((float) (x))
#define ENVF(x) (x)
#define TSC(v, o) dsc(m->tsc[(v) * MAXC + (o)])
#define ESC(v) (m->oesc + (size_t) (v) * Kp * Kp)
#define ESCT float
#define EV(x) dsc(x)
#define BEGINSC(y) dsc(m->beginsc[y])
#define HAS_BEGIN(y) NOT_IMP(m->beginsc[y])
#define ENDSC(v) dsc(m->endsc[v])
#define INIT_SC(v, d) (NOT_IMP(m->endsc[v]) ? (double) m->el_selfsc * (d) + (double) m->endsc[v] : -INFINITY)
#include "cm_scan_oracle_core.h"

/* One scan of dsq[i0..j0].  algo: ORC_CYK (FastCYKScan), ORC_IINS
 * (FastIInsideScan) or ORC_FINS (FastFInsideScan).  Hits go to hits_out
 * (at most max_hits, *ret_nhits = total).  Returns CMGB_OK or an error code. */
int oracle_scan(const cmgb_model_desc *m, int algo, int qdbidx,
                const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                int do_null3, float env_cutoff, int want_hits,
                cmgb_hit *hits_out, int64_t max_hits, int64_t *ret_nhits,
                int64_t *ret_envi, int64_t *ret_envj, float *vsc_out, float *ret_sc,
                char *errbuf)
{
  init_tables();
  if (j0 < i0) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: j0 < i0"); return CMGB_EINCOMPAT; }
  if (dsq == NULL) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: dsq is NULL"); return CMGB_EINCOMPAT; }
  scanctx c;
  memset(&c, 0, sizeof(c));
  c.m = m; c.dsq = dsq; c.i0 = i0; c.j0 = j0; c.L = j0 - i0 + 1;
  c.M = m->M; c.Wm = m->W; c.Kp = m->Kp; c.K = m->K;
  c.W = (int) (c.Wm > c.L ? c.L : c.Wm);     /* local W (src/cm_dpsearch.c:157-158) */
  c.WP = c.Wm + 1;
  if (qdbidx == CMGB_QDB1_TIGHT) { c.dmin = m->dmin1; c.dmax = m->dmax1; }
  else if (qdbidx == CMGB_QDB2_LOOSE) { c.dmin = m->dmin2; c.dmax = m->dmax2; }
  else if (qdbidx != CMGB_NOQDB) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: bad qdbidx"); return CMGB_EINCOMPAT; }
  for (int v = 0; v < m->M; v++)
    if (m->sttype[v] != CMGB_E_st && m->sttype[v] != CMGB_B_st && v > 0 && m->stid[v] != CMGB_BEGL_S && (m->cnum[v] < 2 || m->cnum[v] > 6)) {
      if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: state %d has %d children", v, m->cnum[v]);
      return CMGB_EINCOMPAT;
    }
  /* bands (src/cm_mx.c:5725-5738) */
  c.dn = malloc(sizeof(int) * c.M); c.dxW = malloc(sizeof(int) * c.M);
  for (int v = 0; v < c.M; v++) {
    int lo = m->sttype[v] == CMGB_MP_st ? 2 : 1;
    if (c.dmin) lo = MAXF(c.dmin[v], lo);
    c.dn[v]  = MINF(lo, c.Wm);
    c.dxW[v] = c.dmax ? MINF(c.dmax[v], c.Wm) : c.Wm;
  }
  c.beglidx = malloc(sizeof(int) * c.M);
  for (int v = 0; v < c.M; v++) c.beglidx[v] = (m->stid[v] == CMGB_BEGL_S) ? c.nbegl++ : -1;
  c.cutoff = cutoff; c.env_cutoff = env_cutoff; c.want_hits = want_hits;
  c.vsc = malloc(sizeof(float) * c.M);
  for (int v = 0; v < c.M; v++) c.vsc[v] = IMP;
  c.vsc_root = IMP;
  c.bestf = malloc(sizeof(float) * c.WP); c.bestr = malloc(sizeof(int) * c.WP);
  c.act = do_null3 ? calloc((size_t) c.W + 1, sizeof(double[8])) : NULL;
  c.gamma_mode = want_hits && (m->flags & CMGB_NOTGREEDY);
  if (c.gamma_mode) {
    c.gmx = malloc(sizeof(float) * (c.L + 1)); c.gback = malloc(sizeof(int64_t) * (c.L + 1));
    c.gsave = malloc(sizeof(float) * (c.L + 1)); c.gr = malloc(sizeof(int) * (c.L + 1));
    c.gmode = malloc(sizeof(int) * (c.L + 1));
    c.gmx[0] = 0.f; c.gback[0] = -1;
  }
  c.envi = j0 + 1; c.envj = i0 - 1;

  if (algo == ORC_IINS) core_iinside(&c);
  else if (algo == ORC_FINS) core_finside(&c);
  else if (algo == ORC_DINS) core_dinside(&c);
  else core_cyk(&c);

  c.vsc[0] = c.vsc_root;
  if (want_hits) {
    if (c.gamma_mode) {
      /* TBackGammaHitMx (src/cm_mx.c:7640-7669) */
      int64_t j = j0;
      while (j >= i0) {
        int64_t jp = j - i0 + 1;
        if (c.gback[jp] == -1) j--;
        else {
          if (c.gsave[jp] >= cutoff) hv_push(&c.fin, c.gback[jp], j, c.gr[jp], CMGB_TRMODE_J, c.gsave[jp]);
          j = c.gback[jp] - 1;
        }
      }
    } else remove_overlaps(&c.tmp, &c.fin);
  }
  *ret_nhits = c.fin.n;
  for (int64_t h = 0; h < c.fin.n && h < max_hits; h++) hits_out[h] = c.fin.h[h];
  if (ret_envi) *ret_envi = (c.envi == j0 + 1) ? -1 : c.envi;
  if (ret_envj) *ret_envj = (c.envj == i0 - 1) ? -1 : c.envj;
  if (vsc_out) memcpy(vsc_out, c.vsc, sizeof(float) * c.M);
  if (ret_sc) *ret_sc = c.vsc_root;
  free(c.dn); free(c.dxW); free(c.beglidx); free(c.vsc);
  free(c.bestf); free(c.bestr); free(c.act); free(c.tmp.h); free(c.fin.h);
  free(c.gmx); free(c.gback); free(c.gsave); free(c.gr); free(c.gmode);
  return CMGB_OK;
}

/* C's float -> int conversion as compiled for x86-64 and aarch64: truncation
 * toward zero, saturating to INT_MIN below the int range (IMPOSSIBLE). */
static inline int float_to_int_c(float x) { return x > -2147483648.0f ? (int) x : (int) 0x80000000; }

/* Truncated scanner cores: CYK (RefTrCYKScan) and integer Inside
 * (RefITrInsideScan). */
#define TR_CORE_NAME tr_core_cyk
#define SCT float
#define IMPV IMP
#define COMB(a, b) MAXF((a), (b))
#define IS_PTY(p) NOT_IMP(p)
#define SCOREF(x) (x)
#define TSC(v, o) m->tsc[(v) * MAXC + (o)]
#define ESC(v) (m->oesc + (size_t) (v) * Kp * Kp)
#define LMESC(v) (m->lmesc + (size_t) (v) * Kp)
#define RMESC(v) (m->rmesc + (size_t) (v) * Kp)
#define PTY(y) (((m->flags & CMGB_LOCAL_BEGIN) ? m->tr_l_pty : m->tr_g_pty)[(size_t) c->pty_idx * M + (y)])
#define ENDSC(v) m->endsc[v]
#define INIT_SC(v, d) (NOT_IMP(m->endsc[v]) ? (float) (m->el_selfsc * (d)) + m->endsc[v] : IMP)
#define RUNNING_VSC 1
#include "cm_tr_oracle_core.h"

#define TR_CORE_NAME tr_core_iinside
#define SCT int
#define IMPV (-INFTY)
#define COMB(a, b) ilogsum((a), (b))
#define IS_PTY(p) ((p) != -INFTY)
#define SCOREF(x) scorify(x)
#define TSC(v, o) m->itsc[(v) * MAXC + (o)]
#define ESC(v) (m->ioesc + (size_t) (v) * Kp * Kp)
#define LMESC(v) (m->ilmesc + (size_t) (v) * Kp)
#define RMESC(v) (m->irmesc + (size_t) (v) * Kp)
#define PTY(y) (((m->flags & CMGB_LOCAL_BEGIN) ? m->tr_il_pty : m->tr_ig_pty)[(size_t) c->pty_idx * M + (y)])
/* the integer matrix's d = 0 cells start from the float endsc converted to
 * int (src/cm_mx.c:6941, 6957), not from iendsc */
#define ENDSC(v) float_to_int_c(m->endsc[v])
#define INIT_SC(v, d) ((m->iendsc[v] != -INFTY) ? m->iel_selfsc * (d) + m->iendsc[v] : -INFTY)
#define RUNNING_VSC 0
#include "cm_tr_oracle_core.h"

/* One truncated scan of dsq[i0..j0] (algo 0: RefTrCYKScan, 1:
 * RefITrInsideScan) for pipeline pass pass_idx (2..5).  Outputs as
 * oracle_scan, plus *ret_mode, the mode of the best-scoring parse. */
int oracle_tr_scan(const cmgb_model_desc *m, int algo, int qdbidx, int pass_idx,
                   const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                   int do_null3, float env_cutoff, int want_hits,
                   cmgb_hit *hits_out, int64_t max_hits, int64_t *ret_nhits,
                   int64_t *ret_envi, int64_t *ret_envj, float *vsc_out, float *ret_sc,
                   int *ret_mode, char *errbuf)
{
  init_tables();
  scanctx c;
  memset(&c, 0, sizeof(c));
  /* cm_TrFillFromPassIdx / cm_tr_penalties_IdxForPass */
  switch (pass_idx) {
  case CMGB_PASS_5P_AND_3P_FORCE: case CMGB_PASS_5P_AND_3P_ANY: c.fill_L = c.fill_R = c.fill_T = 1; c.pty_idx = 0; break;
  case CMGB_PASS_5P_ONLY_FORCE: c.fill_R = 1; c.pty_idx = 1; break;
  case CMGB_PASS_3P_ONLY_FORCE: c.fill_L = 1; c.pty_idx = 2; break;
  default: if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: unexpected pass idx: %d", pass_idx); return CMGB_EINVAL;
  }
  if (j0 < i0) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: j0 < i0"); return CMGB_EINCOMPAT; }
  if (dsq == NULL) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: dsq is NULL"); return CMGB_EINCOMPAT; }
  if (m->tr_g_pty == NULL || m->lmesc == NULL || m->emap_lpos == NULL || m->ndtype == NULL) {
    if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: model has no truncation tables");
    return CMGB_EINCOMPAT;
  }
  c.pass_idx = pass_idx;
  c.m = m; c.dsq = dsq; c.i0 = i0; c.j0 = j0; c.L = j0 - i0 + 1;
  c.M = m->M; c.Wm = m->W; c.Kp = m->Kp; c.K = m->K;
  c.W = (int) (c.Wm > c.L ? c.L : c.Wm);
  c.WP = c.Wm + 1;
  if (qdbidx == CMGB_QDB1_TIGHT) { c.dmin = m->dmin1; c.dmax = m->dmax1; }
  else if (qdbidx == CMGB_QDB2_LOOSE) { c.dmin = m->dmin2; c.dmax = m->dmax2; }
  else if (qdbidx != CMGB_NOQDB) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: bad qdbidx"); return CMGB_EINCOMPAT; }
  /* truncated bands: dn = 1 for every state (src/cm_mx.c:6432-6438) */
  c.dn = malloc(sizeof(int) * c.M); c.dxW = malloc(sizeof(int) * c.M);
  for (int v = 0; v < c.M; v++) { c.dn[v] = 1; c.dxW[v] = c.dmax ? MINF(c.dmax[v], c.Wm) : c.Wm; }
  c.beglidx = malloc(sizeof(int) * c.M);
  for (int v = 0; v < c.M; v++) c.beglidx[v] = (m->stid[v] == CMGB_BEGL_S) ? c.nbegl++ : -1;
  c.cutoff = cutoff; c.env_cutoff = env_cutoff; c.want_hits = want_hits;
  c.vsc = malloc(sizeof(float) * c.M);
  for (int v = 0; v < c.M; v++) c.vsc[v] = IMP;
  c.vsc_root = IMP; c.vmode_root = CMGB_TRMODE_UNKNOWN;
  c.bestf = malloc(sizeof(float) * c.WP); c.bestr = malloc(sizeof(int) * c.WP); c.bestmode = malloc(sizeof(int) * c.WP);
  c.act = do_null3 ? calloc((size_t) c.W + 1, sizeof(double[8])) : NULL;
  c.gamma_mode = want_hits && (m->flags & CMGB_NOTGREEDY);
  if (c.gamma_mode) {
    c.gmx = malloc(sizeof(float) * (c.L + 1)); c.gback = malloc(sizeof(int64_t) * (c.L + 1));
    c.gsave = malloc(sizeof(float) * (c.L + 1)); c.gr = malloc(sizeof(int) * (c.L + 1));
    c.gmode = malloc(sizeof(int) * (c.L + 1));
    c.gmx[0] = 0.f; c.gback[0] = -1;
  }
  c.envi = j0 + 1; c.envj = i0 - 1;

  if (algo == 1) tr_core_iinside(&c);
  else tr_core_cyk(&c);

  c.vsc[0] = c.vsc_root;
  if (want_hits) {
    if (c.gamma_mode) {
      int64_t j = j0;
      while (j >= i0) {
        int64_t jp = j - i0 + 1;
        if (c.gback[jp] == -1) j--;
        else {
          if (c.gsave[jp] >= cutoff) hv_push(&c.fin, c.gback[jp], j, c.gr[jp], c.gmode[jp], c.gsave[jp]);
          j = c.gback[jp] - 1;
        }
      }
    } else remove_overlaps(&c.tmp, &c.fin);
  }
  *ret_nhits = c.fin.n;
  for (int64_t h = 0; h < c.fin.n && h < max_hits; h++) hits_out[h] = c.fin.h[h];
  if (ret_envi) *ret_envi = (c.envi == j0 + 1) ? -1 : c.envi;
  if (ret_envj) *ret_envj = (c.envj == i0 - 1) ? -1 : c.envj;
  if (vsc_out) memcpy(vsc_out, c.vsc, sizeof(float) * c.M);
  if (ret_sc) *ret_sc = c.vsc_root;
  if (ret_mode) *ret_mode = c.vmode_root;
  free(c.dn); free(c.dxW); free(c.beglidx); free(c.vsc);
  free(c.bestf); free(c.bestr); free(c.bestmode); free(c.act); free(c.tmp.h); free(c.fin.h);
  free(c.gmx); free(c.gback); free(c.gsave); free(c.gr); free(c.gmode);
  return CMGB_OK;
}

/* DP cell count (the algorithmic work unit of the scan). */
int64_t oracle_count_cells(const cmgb_model_desc *m, int qdbidx, int64_t L)
{
  const int *dmin = qdbidx == 1 ? m->dmin1 : qdbidx == 2 ? m->dmin2 : NULL;
  const int *dmax = qdbidx == 1 ? m->dmax1 : qdbidx == 2 ? m->dmax2 : NULL;
  int64_t cells = 0;
  int Wl = (int) (m->W > L ? L : m->W);
  for (int v = 0; v < m->M; v++) {
    if (m->sttype[v] == CMGB_E_st) continue;
    int lo = m->sttype[v] == CMGB_MP_st ? 2 : 1;
    if (dmin) lo = MAXF(dmin[v], lo);
    int dn = MINF(lo, m->W), dx = dmax ? MINF(dmax[v], m->W) : m->W;
    for (int64_t jp = 1; jp <= L && jp < Wl; jp++) { int hi = MINF((int) jp, dx); if (hi >= dn) cells += hi - dn + 1; }
    if (L >= Wl) { int hi = MINF(Wl, dx); if (hi >= dn) cells += (int64_t) (hi - dn + 1) * (L - Wl + 1); }
  }
  return cells;
}
