/* ref_harness.c -- drives Infernal's own scanner sources, compiled from the
 * read-only reference tree, on a flat model (cmgb_model_desc).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is part of the parity checker: it is
 * linked with the reference's src/cm_dpsearch.c, src/cm_dpsearch_trunc.c,
 * src/cm_mx.c, src/cm_tophits.c, src/cm_trunc.c and src/logsum.c (built by
 * oracle/build_ref.sh into oracle/_ref/) so that the golden vectors under
 * tests/golden/ are produced by the reference's code itself.  Nothing in the
 * product library links or calls it.
 *
 * Besides the harness entry point it restates the small helpers of
 * src/cm.c, src/cm_parsetree.c, src/errors.c and Easel that the scanner
 * sources call but that cannot be compiled here (Easel is not vendored);
 * each cites the function it stands in for.
 */
#include <stdarg.h>
#include "easel.h"
#include "esl_alphabet.h"
#include "hmmer.h"
#include "infernal.h"
#include "../include/infernal_gb300.h"

/* ------------------------------------------------------------------ */
/* Easel stand-ins                                                      */
/* ------------------------------------------------------------------ */
void esl_vec_FSet(float *v, int64_t n, float x)   { for (int64_t i = 0; i < n; i++) v[i] = x; }
void esl_vec_ISet(int *v, int64_t n, int x)       { for (int64_t i = 0; i < n; i++) v[i] = x; }
void esl_vec_DSet(double *v, int64_t n, double x) { for (int64_t i = 0; i < n; i++) v[i] = x; }
void esl_vec_DCopy(const double *s, int64_t n, double *d) { for (int64_t i = 0; i < n; i++) d[i] = s[i]; }
void esl_vec_FCopy(const float *s, int64_t n, float *d)   { for (int64_t i = 0; i < n; i++) d[i] = s[i]; }
void esl_vec_ICopy(const int *s, int64_t n, int *d)       { for (int64_t i = 0; i < n; i++) d[i] = s[i]; }
/* Compensated (Kahan) summation, as Easel's vector sums. */
float esl_vec_FSum(const float *v, int64_t n)
{
  float sum = 0.f, c = 0.f, y, t;
  for (int64_t i = 0; i < n; i++) { y = v[i] - c; t = sum + y; c = (t - sum) - y; sum = t; }
  return sum;
}
double esl_vec_DSum(const double *v, int64_t n)
{
  double sum = 0., c = 0., y, t;
  for (int64_t i = 0; i < n; i++) { y = v[i] - c; t = sum + y; c = (t - sum) - y; sum = t; }
  return sum;
}
void esl_vec_FNorm(float *v, int64_t n)
{
  float sum = esl_vec_FSum(v, n);
  if (sum != 0.f) for (int64_t i = 0; i < n; i++) v[i] /= sum;
  else            for (int64_t i = 0; i < n; i++) v[i] = 1.f / (float) n;
}
void esl_vec_DNorm(double *v, int64_t n)
{
  double sum = esl_vec_DSum(v, n);
  if (sum != 0.) for (int64_t i = 0; i < n; i++) v[i] /= sum;
  else           for (int64_t i = 0; i < n; i++) v[i] = 1. / (double) n;
}
void esl_vec_FScale(float *v, int64_t n, float x) { for (int64_t i = 0; i < n; i++) v[i] *= x; }
int  esl_abc_XIsCanonical(const ESL_ALPHABET *abc, ESL_DSQ x) { return x < abc->K; }
/* Residue counting: canonical residues count once, degenerate codes spread
 * their weight evenly over the residues they stand for. */
int esl_abc_DCount(const ESL_ALPHABET *abc, double *ct, ESL_DSQ x, double wt)
{
  if (x < abc->K) { ct[x] += wt; return eslOK; }
  if (x >= abc->Kp || abc->degen == NULL || abc->ndegen[x] == 0) return eslOK;
  for (int y = 0; y < abc->K; y++) if (abc->degen[x][y]) ct[y] += wt / (double) abc->ndegen[x];
  return eslOK;
}
void esl_fatal(const char *fmt, ...) { va_list ap; va_start(ap, fmt); vfprintf(stderr, fmt, ap); va_end(ap); exit(1); }

/* ------------------------------------------------------------------ */
/* Infernal helpers that live in files which do not compile here        */
/* ------------------------------------------------------------------ */
/* src/errors.c:56 */
void cm_Fail(char *format, ...) { va_list ap; fprintf(stderr, "\nError: "); va_start(ap, format); vfprintf(stderr, format, ap); va_end(ap); fprintf(stderr, "\n"); exit(1); }
/* src/cm.c:1177-1265: emissions per state type */
int StateDelta(int t)      { return t == MP_st ? 2 : (t == ML_st || t == MR_st || t == IL_st || t == IR_st) ? 1 : 0; }
int StateLeftDelta(int t)  { return (t == MP_st || t == ML_st || t == IL_st) ? 1 : 0; }
int StateRightDelta(int t) { return (t == MP_st || t == MR_st || t == IR_st) ? 1 : 0; }
int Emitmode(int t)
{
  switch (t) { case MP_st: return EMITPAIR; case ML_st: case IL_st: return EMITLEFT; case MR_st: case IR_st: return EMITRIGHT; default: return EMITNONE; }
}
/* src/cm.c:1775 */
int StateIsDetached(CM_t *cm, int v) { return (cm->stid[v + 1] == END_E) ? TRUE : FALSE; }
/* src/cm.c:1578 */
char *MarginalMode(char mode)
{
  switch (mode) { case TRMODE_J: return "Joint"; case TRMODE_L: return "Left"; case TRMODE_R: return "Right"; case TRMODE_T: return "Term"; default: return "Unkwn"; }
}
/* src/cm.c:4225 */
float Scorify(int sc) { return (sc == -INFTY) ? IMPOSSIBLE : ((float) sc / INTSCALE); }
/* src/cm.c:4100-4140: init_sc[v][d] = el_selfsc*d + endsc[v] */
float **FCalcInitDPScores(CM_t *cm)
{
  float *el = malloc(sizeof(float) * (cm->W + 1));
  float **a = malloc(sizeof(float *) * cm->M);
  a[0] = malloc(sizeof(float) * cm->M * (cm->W + 1));
  for (int d = 0; d <= cm->W; d++) el[d] = cm->el_selfsc * d;
  for (int v = 0; v < cm->M; v++) {
    a[v] = a[0] + v * (cm->W + 1);
    if (NOT_IMPOSSIBLE(cm->endsc[v])) for (int d = 0; d <= cm->W; d++) a[v][d] = el[d] + cm->endsc[v];
    else                              for (int d = 0; d <= cm->W; d++) a[v][d] = IMPOSSIBLE;
  }
  free(el);
  return a;
}
/* src/cm.c:4146-4185 */
int **ICalcInitDPScores(CM_t *cm)
{
  int *el = malloc(sizeof(int) * (cm->W + 1));
  int **a = malloc(sizeof(int *) * cm->M);
  a[0] = malloc(sizeof(int) * cm->M * (cm->W + 1));
  for (int d = 0; d <= cm->W; d++) el[d] = cm->iel_selfsc * d;
  for (int v = 0; v < cm->M; v++) {
    a[v] = a[0] + v * (cm->W + 1);
    if (cm->iendsc[v] != -INFTY) for (int d = 0; d <= cm->W; d++) a[v][d] = el[d] + cm->iendsc[v];
    else                         for (int d = 0; d <= cm->W; d++) a[v][d] = -INFTY;
  }
  free(el);
  return a;
}
/* src/cm_parsetree.c:2352-2380 */
void ScoreCorrectionNull3(const ESL_ALPHABET *abc, float *null0, float *comp, int len, float omega, float *ret_sc)
{
  float score = 0.;
  for (int a = 0; a < abc->K; a++) score += sreLOG2(comp[a] / null0[a]) * comp[a] * len;
  score += sreLOG2(omega);
  *ret_sc = LogSum2(0., score);
}

/* src/cm.c:4201 */
int Prob2Score(float p, float null) { if (p == 0.0) return -INFTY; return (int) floor(0.5 + INTSCALE * sreLOG2(p / null)); }
/* src/cm_dpalign_trunc.c:9858 */
int cm_TrFillFromMode(char mode, int *fl, int *fr, int *ft)
{
  int L = FALSE, R = FALSE, T = FALSE;
  switch (mode) {
  case TRMODE_J: break;
  case TRMODE_L: L = TRUE; break;
  case TRMODE_R: R = TRUE; break;
  case TRMODE_T: case TRMODE_UNKNOWN: L = R = T = TRUE; break;
  default: return eslEINVAL;
  }
  if (fl) *fl = L; if (fr) *fr = R; if (ft) *ft = T;
  return eslOK;
}

/* Easel's push-down stacks (esl_stack.c): integers for CreateEmitMap,
 * pointers for BandCalculationEngine's reusable beams. */
struct esl_stack_s { int *idata; void **pdata; int n, nalloc; };
ESL_STACK *esl_stack_ICreate(void)
{
  ESL_STACK *s = calloc(1, sizeof(ESL_STACK));
  s->nalloc = 128; s->idata = malloc(sizeof(int) * s->nalloc);
  return s;
}
ESL_STACK *esl_stack_PCreate(void)
{
  ESL_STACK *s = calloc(1, sizeof(ESL_STACK));
  s->nalloc = 128; s->pdata = malloc(sizeof(void *) * s->nalloc);
  return s;
}
int esl_stack_PPush(ESL_STACK *s, void *p)
{
  if (s->n == s->nalloc) { s->nalloc *= 2; s->pdata = realloc(s->pdata, sizeof(void *) * s->nalloc); }
  s->pdata[s->n++] = p;
  return eslOK;
}
int esl_stack_PPop(ESL_STACK *s, void **ret_p)
{
  if (s->n == 0) { *ret_p = NULL; return eslEOD; }
  *ret_p = s->pdata[--s->n];
  return eslOK;
}
int esl_stack_IPush(ESL_STACK *s, int x)
{
  if (s->n == s->nalloc) { s->nalloc *= 2; s->idata = realloc(s->idata, sizeof(int) * s->nalloc); }
  s->idata[s->n++] = x;
  return eslOK;
}
int esl_stack_IPop(ESL_STACK *s, int *ret_x)
{
  if (s->n == 0) { *ret_x = 0; return eslEOD; }
  *ret_x = s->idata[--s->n];
  return eslOK;
}
void esl_stack_Destroy(ESL_STACK *s) { if (s) { free(s->idata); free(s->pdata); free(s); } }

/* src/cm.c:4897 */
void InsertsGivenNodeIndex(CM_t *cm, int nd, int *ret_i1, int *ret_i2)
{
  int i1 = -1, i2 = -1, v = cm->nodemap[nd];
  switch (cm->ndtype[nd]) {
  case MATP_nd: i1 = v + 4; i2 = v + 5; break;
  case MATL_nd: i1 = v + 2; break;
  case MATR_nd: i1 = v + 2; break;
  case BEGR_nd: i1 = v + 1; break;
  case ROOT_nd: i1 = v + 1; i2 = v + 2; break;
  }
  *ret_i1 = i1; *ret_i2 = i2;
}

/* src/cm.c:4250-4330 cm_ExpectedStateOccupancy and src/cm.c:4405
 * cm_ExpectedPositionOccupancy, for a CM without local begins or ends (the
 * state cm_tr_penalties_Create sees during cm_Configure).  The reference
 * looks the parent->child transition up in its transition map; the map's
 * entry for parent x and child v is v's offset in x's child list,
 * v - cfirst[x], which is what is used here. */
int cm_ExpectedPositionOccupancy(CM_t *cm, float **ret_mexpocc, float **ret_iexpocc, double **opt_psi,
                                 int **opt_m2v_1, int **opt_m2v_2, int **opt_i2v)
{
  double *psi = calloc(cm->M, sizeof(double));
  for (int v = 0; v < cm->M; v++) {
    int is_insert = (cm->sttype[v] == IL_st || cm->sttype[v] == IR_st);
    if (cm->sttype[v] == S_st) { psi[v] = 1.0; continue; }
    for (int y = cm->pnum[v] - 1; y >= (is_insert ? 1 : 0); y--) {
      int x = cm->plast[v] - y;
      psi[v] += psi[x] * cm->t[x][v - cm->cfirst[x]];
    }
    if (is_insert) psi[v] += psi[v] * (cm->t[v][0] / (1. - cm->t[v][0]));
  }
  float *mexpocc = calloc(cm->clen + 1, sizeof(float)), *iexpocc = calloc(cm->clen + 1, sizeof(float));
  for (int v = 0; v < cm->M; v++) {
    if (StateIsDetached(cm, v)) continue;
    int nd = cm->ndidx[v], lpos = cm->emap->lpos[nd], rpos = cm->emap->rpos[nd];
    if (cm->sttype[v] == MP_st || cm->sttype[v] == ML_st) mexpocc[lpos] += psi[v];
    if (cm->sttype[v] == MP_st || cm->sttype[v] == MR_st) mexpocc[rpos] += psi[v];
    if (cm->sttype[v] == IL_st) iexpocc[lpos] = psi[v];
    if (cm->sttype[v] == IR_st) iexpocc[rpos - 1] = psi[v];
  }
  *ret_mexpocc = mexpocc; *ret_iexpocc = iexpocc;
  if (opt_psi) *opt_psi = psi; else free(psi);
  if (opt_m2v_1) *opt_m2v_1 = NULL;
  if (opt_m2v_2) *opt_m2v_2 = NULL;
  if (opt_i2v) *opt_i2v = NULL;
  return eslOK;
}

/* ------------------------------------------------------------------ */
/* RNA alphabet (Easel's eslRNA: "ACGU-RYMKSWHBVDN*~")                   */
/* ------------------------------------------------------------------ */
static const char *rna_degen_sets[18] = {
  "A", "C", "G", "U", "", "AG", "CU", "AC", "GU", "CG", "AU", "ACU", "CGU", "ACG", "AGU", "ACGU", "", ""
};
static ESL_ALPHABET *make_rna_alphabet(void)
{
  ESL_ALPHABET *abc = calloc(1, sizeof(ESL_ALPHABET));
  abc->type = eslRNA; abc->K = 4; abc->Kp = 18;
  strcpy(abc->sym, "ACGU-RYMKSWHBVDN*~");
  abc->degen  = malloc(sizeof(char *) * 18);
  abc->ndegen = calloc(18, sizeof(int));
  for (int x = 0; x < 18; x++) {
    abc->degen[x] = calloc(4, 1);
    for (const char *p = rna_degen_sets[x]; *p; p++) {
      int y = (int)(strchr("ACGU", *p) - "ACGU");
      abc->degen[x][y] = 1; abc->ndegen[x]++;
    }
  }
  return abc;
}

/* ------------------------------------------------------------------ */
/* CM_t construction from the flat description                          */
/* ------------------------------------------------------------------ */
static CM_t *build_cm(const cmgb_model_desc *m, int nodes)
{
  int M = m->M, Kp = m->Kp;
  CM_t *cm = calloc(1, sizeof(CM_t));
  cm->M = M; cm->W = m->W; cm->clen = m->clen; cm->nodes = nodes;
  cm->abc = make_rna_alphabet();
  cm->sttype = malloc(M + 1); cm->stid = malloc(M + 1);
  cm->cfirst = malloc(sizeof(int) * M); cm->cnum = malloc(sizeof(int) * M);
  cm->ndidx = calloc(M, sizeof(int));
  for (int v = 0; v < M; v++) {
    cm->sttype[v] = m->sttype[v]; cm->stid[v] = m->stid[v];
    cm->cfirst[v] = m->cfirst[v]; cm->cnum[v] = m->cnum[v];
    if (m->ndidx) cm->ndidx[v] = m->ndidx[v];
  }
  cm->ndtype = calloc(nodes + 1, 1);
  if (m->ndtype) for (int nd = 0; nd < nodes; nd++) cm->ndtype[nd] = m->ndtype[nd];
  cm->sttype[M] = cm->stid[M] = -1;
  cm->qdbinfo = calloc(1, sizeof(CM_QDBINFO));
  cm->qdbinfo->M = M;
  cm->qdbinfo->dmin1 = (int *) m->dmin1; cm->qdbinfo->dmax1 = (int *) m->dmax1;
  cm->qdbinfo->dmin2 = (int *) m->dmin2; cm->qdbinfo->dmax2 = (int *) m->dmax2;
  cm->qdbinfo->setby = CM_QDBINFO_SETBY_CMFILE;
  cm->tsc = malloc(sizeof(float *) * M);  cm->itsc = malloc(sizeof(int *) * M);
  cm->oesc = malloc(sizeof(float *) * M); cm->ioesc = malloc(sizeof(int *) * M);
  cm->lmesc = malloc(sizeof(float *) * M); cm->rmesc = malloc(sizeof(float *) * M);
  cm->ilmesc = malloc(sizeof(int *) * M); cm->irmesc = malloc(sizeof(int *) * M);
  for (int v = 0; v < M; v++) {
    cm->tsc[v]  = (float *) m->tsc  + (size_t) v * 6;
    cm->itsc[v] = (int *)   m->itsc + (size_t) v * 6;
    cm->oesc[v]  = (float *) m->oesc  + (size_t) v * Kp * Kp;
    cm->ioesc[v] = (int *)   m->ioesc + (size_t) v * Kp * Kp;
    if (m->lmesc) {
      cm->lmesc[v]  = (float *) m->lmesc  + (size_t) v * Kp; cm->rmesc[v]  = (float *) m->rmesc  + (size_t) v * Kp;
      cm->ilmesc[v] = (int *)   m->ilmesc + (size_t) v * Kp; cm->irmesc[v] = (int *)   m->irmesc + (size_t) v * Kp;
    }
  }
  cm->endsc = (float *) m->endsc; cm->beginsc = (float *) m->beginsc;
  cm->iendsc = (int *) m->iendsc; cm->ibeginsc = (int *) m->ibeginsc;
  cm->el_selfsc = m->el_selfsc; cm->iel_selfsc = m->iel_selfsc;
  cm->null = (float *) m->null; cm->null3_omega = m->null3_omega;
  cm->flags = CMH_BITS;
  if (m->flags & CMGB_LOCAL_BEGIN) cm->flags |= CMH_LOCAL_BEGIN;
  if (m->flags & CMGB_LOCAL_END)   cm->flags |= CMH_LOCAL_END;
  cm->search_opts = 0;
  if (m->flags & CMGB_NOTGREEDY) cm->search_opts |= CM_SEARCH_CMNOTGREEDY;
  if (m->tr_g_pty) {
    CM_TR_PENALTIES *trp = calloc(1, sizeof(CM_TR_PENALTIES));
    trp->M = M;
    trp->g_ptyAA  = malloc(sizeof(float *) * NTRPENALTY); trp->l_ptyAA  = malloc(sizeof(float *) * NTRPENALTY);
    trp->ig_ptyAA = malloc(sizeof(int *) * NTRPENALTY);   trp->il_ptyAA = malloc(sizeof(int *) * NTRPENALTY);
    for (int p = 0; p < NTRPENALTY; p++) {
      trp->g_ptyAA[p]  = (float *) m->tr_g_pty  + (size_t) p * M; trp->l_ptyAA[p]  = (float *) m->tr_l_pty  + (size_t) p * M;
      trp->ig_ptyAA[p] = (int *)   m->tr_ig_pty + (size_t) p * M; trp->il_ptyAA[p] = (int *)   m->tr_il_pty + (size_t) p * M;
    }
    cm->trp = trp;
  }
  if (m->emap_lpos) {
    CMEmitMap_t *emap = calloc(1, sizeof(CMEmitMap_t));
    emap->clen = m->clen;
    emap->lpos = (int *) m->emap_lpos; emap->rpos = (int *) m->emap_rpos;
    cm->emap = emap;
  }
  return cm;
}

/* Algorithms the harness can run. */
enum { REFH_FASTCYK = 0, REFH_REFCYK = 1, REFH_FASTIINS = 2, REFH_REFIINS = 3,
       REFH_FASTFINS = 4, REFH_REFFINS = 5, REFH_TRCYK = 6, REFH_ITRINS = 7 };

/* Runs one reference scanner over dsq[i0..j0] and copies its outputs.
 * hits_out receives at most max_hits hits in hit-list order; *ret_nhits is
 * the full count.  vsc_out (M floats) may be NULL.  Returns the scanner's
 * status code; errbuf receives its message. */
int refh_scan_full(const cmgb_model_desc *m, int nodes, int algo, int qdbidx,
                   const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                   int do_null3, float env_cutoff, int pass_idx, int want_hits,
                   cmgb_hit *hits_out, int64_t max_hits, int64_t *ret_nhits,
                   int64_t *ret_envi, int64_t *ret_envj, float *vsc_out, float *ret_sc,
                   int *ret_mode, int64_t *extra_out, char *errbuf);

int refh_scan(const cmgb_model_desc *m, int nodes, int algo, int qdbidx,
              const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
              int do_null3, float env_cutoff, int pass_idx, int want_hits,
              cmgb_hit *hits_out, int64_t max_hits, int64_t *ret_nhits,
              int64_t *ret_envi, int64_t *ret_envj, float *vsc_out, float *ret_sc,
              int *ret_mode, char *errbuf)
{
  return refh_scan_full(m, nodes, algo, qdbidx, dsq, i0, j0, cutoff, do_null3, env_cutoff, pass_idx, want_hits,
                        hits_out, max_hits, ret_nhits, ret_envi, ret_envj, vsc_out, ret_sc, ret_mode, NULL, errbuf);
}

/* As refh_scan; extra_out (when not NULL) receives, per hit, the other
 * CM_HIT fields a scanner call leaves behind, as REFH_NEXTRA integers:
 * srcL, flags, hit_idx, hmmonly, cm_idx, seq_idx, pass_idx, in_rc, glocal,
 * has_evalue, and the bit patterns of pvalue and evalue (doubles). */
#define REFH_NEXTRA 12
int refh_scan_full(const cmgb_model_desc *m, int nodes, int algo, int qdbidx,
                   const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                   int do_null3, float env_cutoff, int pass_idx, int want_hits,
                   cmgb_hit *hits_out, int64_t max_hits, int64_t *ret_nhits,
                   int64_t *ret_envi, int64_t *ret_envj, float *vsc_out, float *ret_sc,
                   int *ret_mode, int64_t *extra_out, char *errbuf)
{
  static int tables_ready = 0;
  if (!tables_ready) { init_ilogsum(); FLogsumInit(); tables_ready = 1; }
  int status;
  CM_t *cm = build_cm(m, nodes);
  CM_SCAN_MX *smx = NULL;
  CM_TR_SCAN_MX *trsmx = NULL;
  CM_TOPHITS *th = want_hits ? cm_tophits_Create() : NULL;
  float *vsc = NULL, sc = 0.f;
  char mode = TRMODE_J;
  int64_t envi = -1, envj = -1;
  ESL_DSQ *q = (ESL_DSQ *) dsq;
  if (algo == REFH_FASTIINS || algo == REFH_REFIINS || algo == REFH_ITRINS ||
      algo == REFH_FASTFINS || algo == REFH_REFFINS)
    cm->search_opts |= CM_SEARCH_INSIDE;
  if (algo >= REFH_TRCYK) {
    if ((status = cm_tr_scan_mx_Create(cm, errbuf, TRUE, TRUE, &trsmx)) != eslOK) return status;
  } else {
    if ((status = cm_scan_mx_Create(cm, errbuf, TRUE, TRUE, &smx)) != eslOK) return status;
  }
  switch (algo) {
  case REFH_FASTCYK: status = FastCYKScan    (cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_REFCYK:  status = RefCYKScan     (cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_FASTIINS:status = FastIInsideScan(cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_REFIINS: status = RefIInsideScan (cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_FASTFINS:status = FastFInsideScan(cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_REFFINS: status = RefFInsideScan (cm, errbuf, smx, qdbidx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &sc); break;
  case REFH_TRCYK:   status = RefTrCYKScan   (cm, errbuf, trsmx, qdbidx, pass_idx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &mode, &sc); break;
  case REFH_ITRINS:  status = RefITrInsideScan(cm, errbuf, trsmx, qdbidx, pass_idx, q, i0, j0, cutoff, th, do_null3, env_cutoff, &envi, &envj, &vsc, &mode, &sc); break;
  default: status = eslEINVAL; break;
  }
  if (status == eslOK) {
    if (th) {
      *ret_nhits = (int64_t) th->N;
      for (int64_t h = 0; h < (int64_t) th->N && h < max_hits; h++) {
        hits_out[h].start = th->unsrt[h].start; hits_out[h].stop = th->unsrt[h].stop;
        hits_out[h].root  = th->unsrt[h].root;  hits_out[h].mode = th->unsrt[h].mode;
        hits_out[h].score = th->unsrt[h].score;
        if (extra_out) {
          const CM_HIT *x = &th->unsrt[h];
          int64_t *e = extra_out + h * REFH_NEXTRA;
          e[0] = x->srcL; e[1] = x->flags; e[2] = x->hit_idx; e[3] = x->hmmonly; e[4] = x->cm_idx; e[5] = x->seq_idx;
          e[6] = x->pass_idx; e[7] = x->in_rc; e[8] = x->glocal; e[9] = x->has_evalue;
          memcpy(&e[10], &x->pvalue, sizeof(double)); memcpy(&e[11], &x->evalue, sizeof(double));
        }
      }
    } else *ret_nhits = 0;
    if (vsc_out && vsc) memcpy(vsc_out, vsc, sizeof(float) * m->M);
    *ret_envi = envi; *ret_envj = envj; *ret_sc = sc; *ret_mode = (int) mode;
  }
  free(vsc);
  if (th) cm_tophits_Destroy(th);
  /* the scan matrices and CM shell are leaked deliberately: the harness runs
   * a handful of scans per process and their destructors touch fields this
   * shell never allocates. */
  return status;
}

/* Truncation penalties and emit map of a CM, computed by the reference's own
 * cm_tr_penalties_Create (src/cm_trunc.c:51), CreateEmitMap
 * (src/display.c:1110) and cm_CalculateLocalBeginProbs
 * (src/cm_modelconfig.c:397), on the renormalised global transition
 * probabilities t[M*6].  Outputs: lpos/rpos[nodes]; g/l/ig/il[3*M] indexed
 * [pty_idx*M + v]. */
int refh_tr_penalties(int M, int nodes, int clen, const int8_t *sttype, const int8_t *stid,
                      const int *ndidx, const int *cfirst, const int *cnum, const int *plast,
                      const int *pnum, const int8_t *ndtype, const int *nodemap, const float *t,
                      float pbegin, int *lpos_out, int *rpos_out, float *g_out, float *l_out,
                      int *ig_out, int *il_out, char *errbuf)
{
  CM_t *cm = calloc(1, sizeof(CM_t));
  cm->M = M; cm->nodes = nodes; cm->clen = clen; cm->pbegin = pbegin;
  cm->sttype = malloc(M + 1); cm->stid = malloc(M + 1);
  cm->ndidx = malloc(sizeof(int) * M); cm->cfirst = malloc(sizeof(int) * M); cm->cnum = malloc(sizeof(int) * M);
  cm->plast = malloc(sizeof(int) * M); cm->pnum = malloc(sizeof(int) * M);
  cm->ndtype = malloc(nodes + 1); cm->nodemap = malloc(sizeof(int) * nodes);
  cm->t = malloc(sizeof(float *) * M);
  for (int v = 0; v < M; v++) {
    cm->sttype[v] = sttype[v]; cm->stid[v] = stid[v]; cm->ndidx[v] = ndidx[v];
    cm->cfirst[v] = cfirst[v]; cm->cnum[v] = cnum[v]; cm->plast[v] = plast[v]; cm->pnum[v] = pnum[v];
    cm->t[v] = (float *) t + (size_t) v * MAXCONNECT;
  }
  cm->sttype[M] = cm->stid[M] = -1;
  for (int nd = 0; nd < nodes; nd++) { cm->ndtype[nd] = ndtype[nd]; cm->nodemap[nd] = nodemap[nd]; }
  cm->ndtype[nodes] = -1;
  if ((cm->emap = CreateEmitMap(cm)) == NULL) { snprintf(errbuf, 128, "CreateEmitMap failed"); return eslFAIL; }
  CM_TR_PENALTIES *trp = cm_tr_penalties_Create(cm, FALSE, errbuf);
  if (trp == NULL) { snprintf(errbuf, 128, "cm_tr_penalties_Create failed"); return eslFAIL; }
  for (int nd = 0; nd < nodes; nd++) { lpos_out[nd] = cm->emap->lpos[nd]; rpos_out[nd] = cm->emap->rpos[nd]; }
  for (int p = 0; p < NTRPENALTY; p++)
    for (int v = 0; v < M; v++) {
      g_out[p * M + v] = trp->g_ptyAA[p][v];  l_out[p * M + v] = trp->l_ptyAA[p][v];
      ig_out[p * M + v] = trp->ig_ptyAA[p][v]; il_out[p * M + v] = trp->il_ptyAA[p][v];
    }
  return eslOK;
}

/* Query-dependent bands and W computed by the reference's own
 * CalculateQueryDependentBands / BandCalculationEngine (src/cm_qdband.c:45,
 * 163) on the renormalised global transition probabilities t[M*6], with
 * local begin probabilities from pbegin (cm_CalculateLocalBeginProbs,
 * compiled from src/cm_modelconfig.c).  Outputs dmin1/dmax1/dmin2/dmax2[M]
 * and *ret_W. */
int refh_qdb_bands(int M, int nodes, int clen, const int8_t *sttype, const int8_t *stid, const int *cfirst,
                   const int *cnum, const int *pnum, const int8_t *ndtype, const int *nodemap, const float *t,
                   float pbegin, double beta1, double beta2, double beta_W,
                   int *dmin1, int *dmax1, int *dmin2, int *dmax2, int *ret_W, char *errbuf)
{
  CM_t *cm = calloc(1, sizeof(CM_t));
  cm->M = M; cm->nodes = nodes; cm->clen = clen; cm->pbegin = pbegin;
  cm->sttype = malloc(M + 1); cm->stid = malloc(M + 1);
  cm->cfirst = malloc(sizeof(int) * M); cm->cnum = malloc(sizeof(int) * M); cm->pnum = malloc(sizeof(int) * M);
  cm->ndtype = malloc(nodes + 1); cm->nodemap = malloc(sizeof(int) * nodes);
  cm->t = malloc(sizeof(float *) * M);
  cm->t[0] = malloc(sizeof(float) * M * MAXCONNECT);
  cm->begin = calloc(M, sizeof(float));
  for (int v = 0; v < M; v++) {
    cm->sttype[v] = sttype[v]; cm->stid[v] = stid[v];
    cm->cfirst[v] = cfirst[v]; cm->cnum[v] = cnum[v]; cm->pnum[v] = pnum[v];
    cm->t[v] = cm->t[0] + (size_t) v * MAXCONNECT;
    for (int x = 0; x < MAXCONNECT; x++) cm->t[v][x] = t[(size_t) v * MAXCONNECT + x];
  }
  cm->sttype[M] = cm->stid[M] = -1;
  for (int nd = 0; nd < nodes; nd++) { cm->ndtype[nd] = ndtype[nd]; cm->nodemap[nd] = nodemap[nd]; }
  cm->ndtype[nodes] = -1;
  CM_QDBINFO *q = calloc(1, sizeof(CM_QDBINFO));
  q->M = M; q->beta1 = beta1; q->beta2 = beta2;
  q->dmin1 = dmin1; q->dmax1 = dmax1; q->dmin2 = dmin2; q->dmax2 = dmax2;
  int status = CalculateQueryDependentBands(cm, errbuf, q, beta_W, ret_W, NULL, NULL, NULL);
  return status;
}
