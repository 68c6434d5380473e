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
 *   remove_overlaps()     cm_tophits_SortForOverlapRemoval + RemoveOrMarkOverlaps
 *                         src/cm_tophits.c:220-245, 400, 1097-1275
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

enum { ORC_CYK = 0, ORC_IINS = 1, ORC_FINS = 2 };

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
typedef union { float f; int i; } cell;

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
  const int M = m->M, Wm = m->W, Kp = m->Kp, K = m->K;
  const int isint = (algo == ORC_IINS);
  const int64_t L = j0 - i0 + 1;
  const int W = (int) (Wm > L ? L : Wm);     /* local W (src/cm_dpsearch.c:157-158) */
  const int *dmin = NULL, *dmax = NULL;
  if (qdbidx == CMGB_QDB1_TIGHT) { dmin = m->dmin1; dmax = m->dmax1; }
  else if (qdbidx == CMGB_QDB2_LOOSE) { dmin = m->dmin2; dmax = m->dmax2; }
  else if (qdbidx != CMGB_NOQDB) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: bad qdbidx"); return CMGB_EINCOMPAT; }

  /* bands (src/cm_mx.c:5725-5738) */
  int *dn = malloc(sizeof(int) * M), *dxW = malloc(sizeof(int) * M);
  for (int v = 0; v < M; v++) {
    int lo = m->sttype[v] == CMGB_MP_st ? 2 : 1;
    if (dmin) lo = MAXF(dmin[v], lo);
    dn[v]  = MINF(lo, Wm);
    dxW[v] = dmax ? MINF(dmax[v], Wm) : Wm;
  }
  /* matrices: alpha[2][M][W+1], begl[W+1][M][W+1] (only BEGL rows used) */
  const int WP = Wm + 1;
  cell *alpha = malloc(sizeof(cell) * 2 * (size_t) M * WP);
  int nbegl = 0;
  int *beglidx = malloc(sizeof(int) * M);
  for (int v = 0; v < M; v++) beglidx[v] = (m->stid[v] == CMGB_BEGL_S) ? nbegl++ : -1;
  cell *begl = malloc(sizeof(cell) * (size_t) (W + 1) * (nbegl ? nbegl : 1) * WP);
  cell impv; if (isint) impv.i = -INFTY; else impv.f = IMP;
  for (size_t k = 0; k < 2 * (size_t) M * WP; k++) alpha[k] = impv;
  for (size_t k = 0; k < (size_t) (W + 1) * (nbegl ? nbegl : 1) * WP; k++) begl[k] = impv;
#define A(r, v, d)  alpha[((size_t) (r) * M + (v)) * WP + (d)]
#define BG(r, b, d) begl[((size_t) (r) * (nbegl ? nbegl : 1) + (b)) * WP + (d)]
  /* d = 0 initialisation (src/cm_mx.c:6039-6138) */
  for (int v = M - 1; v >= 0; v--) {
    int t = m->sttype[v], y = m->cfirst[v];
    cell c = impv;
    if (m->stid[v] == CMGB_BEGL_S || t == CMGB_S_st || t == CMGB_D_st) {
      if (isint) {
        int s = m->iendsc[v];
        for (int o = 0; o < m->cnum[v]; o++) { int cand = A(0, y + o, 0).i + m->itsc[v * MAXC + o]; s = s > cand ? s : cand; }
        c.i = s > -INFTY ? s : -INFTY;
      } else {
        float s = m->endsc[v];
        for (int o = 0; o < m->cnum[v]; o++) s = MAXF(s, A(0, y + o, 0).f + m->tsc[v * MAXC + o]);
        c.f = MAXF(s, IMP);
      }
    } else if (t == CMGB_E_st) {
      if (isint) c.i = 0; else c.f = 0.f;
    } else if (t == CMGB_B_st) {
      int w = m->cfirst[v], yy = m->cnum[v];
      if (isint) c.i = BG(0, beglidx[w], 0).i + A(0, yy, 0).i;
      else       c.f = BG(0, beglidx[w], 0).f + A(0, yy, 0).f;
    }
    if (m->stid[v] == CMGB_BEGL_S) { for (int r = 0; r <= W; r++) BG(r, beglidx[v], 0) = c; }
    else { A(0, v, 0) = c; A(1, v, 0) = c; }
  }
  /* init scores (src/cm.c:4100-4185) */
  cell *init = malloc(sizeof(cell) * (size_t) M * WP);
  for (int v = 0; v < M; v++)
    for (int d = 0; d <= Wm; d++) {
      if (isint) init[(size_t) v * WP + d].i = (m->iendsc[v] != -INFTY) ? m->iel_selfsc * d + m->iendsc[v] : -INFTY;
      else { float el = m->el_selfsc * d; init[(size_t) v * WP + d].f = NOT_IMP(m->endsc[v]) ? el + m->endsc[v] : IMP; }
    }
#define INIT(v, d) init[(size_t) (v) * WP + (d)]

  float *vsc = malloc(sizeof(float) * M);
  for (int v = 0; v < M; v++) vsc[v] = IMP;
  float vsc_root = IMP;
  cell *bestsc = malloc(sizeof(cell) * WP);
  int *bestr = malloc(sizeof(int) * WP);
  float *bestf = malloc(sizeof(float) * WP);
  double (*act)[8] = do_null3 ? calloc((size_t) W + 1, sizeof(double[8])) : NULL;
  int gamma_mode = want_hits && (m->flags & CMGB_NOTGREEDY);
  float *gmx = NULL; int64_t *gback = NULL; float *gsave = NULL; int *gr = NULL;
  if (gamma_mode) {
    gmx = malloc(sizeof(float) * (L + 1)); gback = malloc(sizeof(int64_t) * (L + 1));
    gsave = malloc(sizeof(float) * (L + 1)); gr = malloc(sizeof(int) * (L + 1));
    gmx[0] = 0.f; gback[0] = -1;
  }
  hitvec tmp = {0}, fin = {0};
  int64_t envi = j0 + 1, envj = i0 - 1;

  for (int64_t j = i0; j <= j0; j++) {
    const int64_t jp = j - i0 + 1;
    const int cur = (int) (j % 2), prv = (int) ((j - 1) % 2);
    const int jrow = (int) (j % (W + 1));
    int jr = jp >= W ? W : (int) jp;  /* band row */
    if (act) {
      memcpy(act[jp % (W + 1)], act[(jp - 1) % (W + 1)], sizeof(double[8]));
      count_residue(act[jp % (W + 1)], dsq[j], K);
    }
    for (int v = M - 1; v > 0; v--) {
      const int t = m->sttype[v];
      if (t == CMGB_E_st) continue;
      const int sd = st_delta(t), cnum = m->cnum[v], y0 = m->cfirst[v];
      const int dnv = dn[v], dxv = MINF(jr, dxW[v]);
      const int jpy = st_right(t) ? prv : cur;
      const int isbegl = (m->stid[v] == CMGB_BEGL_S);
      const float *tsc = m->tsc + v * MAXC; const int *itsc = m->itsc + v * MAXC;
      const float *esc = m->oesc + (size_t) v * Kp * Kp; const int *iesc = m->ioesc + (size_t) v * Kp * Kp;
      for (int d = dnv; d <= dxv; d++) {
        cell sc;
        const int dp = d - sd;
        if (t == CMGB_B_st) {
          int w = m->cfirst[v], yy = m->cnum[v], kmin, kmax;
          if (dmin) {
            int dny = MINF(dmin[yy], Wm), dxy = MINF(dmax[yy], Wm), dnw = MINF(dmin[w], Wm), dxw = MINF(dmax[w], Wm);
            kmin = MAXF(0, MAXF(dny, d - dxw)); kmax = MINF(dxy, d - dnw);
          } else { kmin = 0; kmax = d; }
          sc = INIT(v, dp);
          for (int k = kmin; k <= kmax; k++) {
            int br = (int) ((j - k) % (W + 1));
            if (isint) sc.i = ilogsum(sc.i, BG(br, beglidx[w], d - k).i + A(cur, yy, k).i);
            else if (algo == ORC_FINS) sc.f = flogsum(sc.f, BG(br, beglidx[w], d - k).f + A(cur, yy, k).f);
            else sc.f = MAXF(sc.f, BG(br, beglidx[w], d - k).f + A(cur, yy, k).f);
          }
        } else if (isbegl) {
          sc = INIT(v, dp);
          for (int o = 0; o < cnum; o++) {
            if (isint) sc.i = ilogsum(sc.i, A(jpy, y0 + o, dp).i + itsc[o]);
            else if (algo == ORC_FINS) sc.f = flogsum(sc.f, A(jpy, y0 + o, dp).f + tsc[o]);
            else sc.f = MAXF(sc.f, A(jpy, y0 + o, dp).f + tsc[o]);
          }
        } else {
          /* the Fast scanners' fold order per child count (src/cm_dpsearch.c:307-519) */
          static const int order[7][7] = {
            {0}, {0}, {1, -1, 0}, {2, 1, -1, 0}, {3, 2, -1, 1, 0}, {4, 3, -1, 1, 2, 0}, {5, -1, 4, 3, 2, 1, 0} };
          if (cnum < 2 || cnum > 6) { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, "oracle: state %d has %d children", v, cnum); return CMGB_EINCOMPAT; }
          const int *ord = order[cnum];
          for (int q = 0; q <= cnum; q++) {
            cell term;
            if (ord[q] < 0) term = INIT(v, dp);
            else if (isint) term.i = A(jpy, y0 + ord[q], dp).i + itsc[ord[q]];
            else term.f = A(jpy, y0 + ord[q], dp).f + tsc[ord[q]];
            if (q == 0) sc = term;
            else if (isint) sc.i = ilogsum(sc.i, term.i);
            else if (algo == ORC_FINS) sc.f = flogsum(sc.f, term.f);
            else sc.f = MAXF(sc.f, term.f);
          }
          /* emission */
          int64_t i = j - d + 1;
          int e = -1;
          if (t == CMGB_MP_st) e = dsq[i] * Kp + dsq[j];
          else if (st_left(t)) e = dsq[i];
          else if (st_right(t)) e = dsq[j];
          if (e >= 0) { if (isint) sc.i += iesc[e]; else sc.f += esc[e]; }
        }
        if (isbegl) BG(jrow, beglidx[v], d) = sc; else A(cur, v, d) = sc;
        float sf = isint ? scorify(sc.i) : sc.f;
        vsc[v] = MAXF(vsc[v], sf);
      }
    }
    /* root and local begins (src/cm_dpsearch.c:562-616) */
    const int dn0 = dn[0], dx0 = MINF(jr, dxW[0]);
    for (int d = 0; d <= W; d++) { bestr[d] = -1; bestf[d] = IMP; }
    for (int d = dn0; d <= dx0; d++) {
      bestr[d] = 0;
      int y = m->cfirst[0];
      cell r;
      if (isint) {
        int s = A(cur, y, d).i + m->itsc[0]; r.i = s > -INFTY ? s : -INFTY;
        for (int o = 1; o < m->cnum[0]; o++) r.i = ilogsum(r.i, A(cur, y + o, d).i + m->itsc[o]);
      } else {
        r.f = MAXF(IMP, A(cur, y, d).f + m->tsc[0]);
        for (int o = 1; o < m->cnum[0]; o++) {
          if (algo == ORC_FINS) r.f = flogsum(r.f, A(cur, y + o, d).f + m->tsc[o]);
          else r.f = MAXF(r.f, A(cur, y + o, d).f + m->tsc[o]);
        }
      }
      A(cur, 0, d) = r;
    }
    if (m->flags & CMGB_LOCAL_BEGIN) {
      for (int y = 1; y < M; y++) {
        int ok = isint ? (m->ibeginsc[y] != -INFTY) : NOT_IMP(m->beginsc[y]);
        if (!ok) continue;
        int lo = MAXF(dn0, dn[y]), hi = MINF(dx0, MINF(jr, dxW[y]));
        for (int d = lo; d <= hi; d++) {
          cell c = (m->stid[y] == CMGB_BEGL_S) ? BG(jrow, beglidx[y], d) : A(cur, y, d);
          if (isint) { int s = c.i + m->ibeginsc[y]; if (A(cur, 0, d).i < s) { A(cur, 0, d).i = s; bestr[d] = y; } }
          else { float s = c.f + m->beginsc[y]; if (A(cur, 0, d).f < s) { A(cur, 0, d).f = s; bestr[d] = y; } }
        }
      }
    }
    for (int d = dn0; d <= dx0; d++) {
      bestf[d] = isint ? scorify(A(cur, 0, d).i) : A(cur, 0, d).f;
      vsc_root = MAXF(vsc_root, bestf[d]);
      float envsc = isint ? (float) A(cur, 0, d).i : A(cur, 0, d).f;
      if (envsc >= env_cutoff) { if (j - d + 1 < envi) envi = j - d + 1; if (j > envj) envj = j; }
    }
    if (!want_hits || dn0 > dx0) { if (gamma_mode) { gmx[jp] = gmx[jp - 1]; gback[jp] = -1; } continue; }
    if (gamma_mode) {
      /* UpdateGammaHitMx (src/cm_mx.c:7440-7520) */
      gmx[jp] = gmx[jp - 1]; gback[jp] = -1; gsave[jp] = IMP; gr[jp] = -1;
      for (int d = MAXF(1, dn0); d <= dx0; d++) {
        int64_t ip = jp - d + 1;
        float hs = bestf[d], cum = gmx[ip - 1] + hs;
        if (cum > gmx[jp] && NOT_IMP(hs)) {
          int rep = 1;
          if (act) {
            float c3 = null3_correction(m, act[jp % (W + 1)], act[(ip - 1) % (W + 1)], d);
            hs -= c3; cum -= c3; rep = cum > gmx[jp];
          }
          if (rep) { gmx[jp] = cum; gback[jp] = j - d + 1; gsave[jp] = hs; gr[jp] = bestr[d]; }
        }
      }
    } else {
      /* ReportHitsGreedily (src/cm_mx.c:7547-7628) */
      float best = IMP;
      for (int d = MAXF(1, dn0); d <= dx0; d++) {
        float hs = bestf[d];
        if (hs > best && hs >= cutoff && NOT_IMP(hs)) {
          int rep = 1;
          if (act) {
            int64_t ip = jp - d + 1;
            hs -= null3_correction(m, act[jp % (W + 1)], act[(ip - 1) % (W + 1)], d);
            rep = (hs > best && hs >= cutoff);
          }
          if (rep) { hv_push(&tmp, j - d + 1, j, bestr[d], CMGB_TRMODE_J, hs); best = hs; }
        }
      }
    }
  }
  vsc[0] = vsc_root;
  if (want_hits) {
    if (gamma_mode) {
      /* TBackGammaHitMx (src/cm_mx.c:7640-7669) */
      int64_t j = j0;
      while (j >= i0) {
        int64_t jp = j - i0 + 1;
        if (gback[jp] == -1) j--;
        else {
          if (gsave[jp] >= cutoff) hv_push(&fin, gback[jp], j, gr[jp], CMGB_TRMODE_J, gsave[jp]);
          j = gback[jp] - 1;
        }
      }
    } else remove_overlaps(&tmp, &fin);
  }
  *ret_nhits = fin.n;
  for (int64_t h = 0; h < fin.n && h < max_hits; h++) hits_out[h] = fin.h[h];
  if (ret_envi) *ret_envi = (envi == j0 + 1) ? -1 : envi;
  if (ret_envj) *ret_envj = (envj == i0 - 1) ? -1 : envj;
  if (vsc_out) memcpy(vsc_out, vsc, sizeof(float) * M);
  if (ret_sc) *ret_sc = vsc_root;
  free(dn); free(dxW); free(alpha); free(begl); free(beglidx); free(init); free(vsc);
  free(bestsc); free(bestr); free(bestf); free(act); free(tmp.h); free(fin.h);
  free(gmx); free(gback); free(gsave); free(gr);
  return CMGB_OK;
#undef A
#undef BG
#undef INIT
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
