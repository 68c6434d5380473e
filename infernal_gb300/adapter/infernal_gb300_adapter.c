/* infernal_gb300_adapter.c -- Infernal's scanner entry points on the GB300 library.
 *
 * Compiled into an Infernal build in place of the CPU scanners it replaces,
 * this file defines the reference's own symbols with their exact prototypes
 * (src/infernal.h:2710-2725):
 *
 *   FastCYKScan      src/cm_dpsearch.c:90
 *   FastIInsideScan  src/cm_dpsearch.c:1106
 *   FastFInsideScan  src/cm_dpsearch.c:1731
 *   RefTrCYKScan     src/cm_dpsearch_trunc.c:79
 *   RefITrInsideScan src/cm_dpsearch_trunc.c:741
 *
 * and forwards each call to the C ABI of include/infernal_gb300.h.  Build it
 * with Infernal's include paths plus this library's include/ directory, and
 * link Infernal against libinfernal_gb300.so instead of compiling
 * src/cm_dpsearch.c's and src/cm_dpsearch_trunc.c's scanners:
 *
 *   cc -c -I<infernal>/src -I<easel> -I<hmmer>/src -I<this repo>/include \
 *      infernal_gb300_adapter.c
 *
 * What it does per call:
 *   - checks the reference's contract (same conditions, same eslEINCOMPAT
 *     messages in errbuf);
 *   - flattens the configured CM_t into a cmgb_model_desc (exactly the fields
 *     the scanners read: tsc/itsc, oesc/ioesc with their Kp or Kp*Kp rows,
 *     endsc/beginsc, el_selfsc, the QDB bands, the local-mode and greedy
 *     flags, NULL3's background, and for the truncated scanners lmesc/rmesc,
 *     the truncated-begin penalties and the emit map), uploads it once and
 *     keeps it in a small per-thread cache keyed by the CM_t's address and a
 *     signature of its configuration (a reconfigured CM gets a new upload);
 *   - scans on this thread's device context (one per host thread, as every
 *     Infernal worker keeps its own CM_SCAN_MX; device 0, or the index in the
 *     environment variable INFERNAL_GB300_DEVICE);
 *   - appends the hits to the caller's CM_TOPHITS through
 *     cm_tophits_CreateNextHit in the reference's order with the fields the
 *     reference sets (greedy resolution copies its non-overlapping hits with
 *     srcL = j0, as cm_tophits_CloneHitMostly does after
 *     cm_tophits_RemoveOrMarkOverlaps; optimal resolution adds them straight
 *     from the gamma traceback), and allocates *ret_vsc (M floats) for the
 *     caller to free.
 * The scan matrices (CM_SCAN_MX / CM_TR_SCAN_MX) are only checked, as the
 * reference checks them: the rolling DP rows live on the GPU.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "easel.h"
#include "esl_alphabet.h"
#include "hmmer.h"
#include "infernal.h"

#include "infernal_gb300.h"

#define ADAPTER_MODELS 8   /* cached model uploads per host thread */

typedef struct {
  const CM_t *cm;
  uint64_t    sig;
  int         tr;          /* uploaded with the truncation tables */
  cmgb_model *model;
} adapter_model_t;

typedef struct {
  cmgb_ctx       *ctx;
  cmgb_hitlist   *hl;
  adapter_model_t models[ADAPTER_MODELS];
  int             next;    /* round-robin eviction */
} adapter_thread_t;

static __thread adapter_thread_t *tls = NULL;

/* FNV-1a over a byte range */
static uint64_t fnv(uint64_t h, const void *p, size_t n)
{
  const unsigned char *b = (const unsigned char *) p;
  for (size_t i = 0; i < n; i++) { h ^= b[i]; h *= 1099511628211ULL; }
  return h;
}

/* Signature of everything a scan reads from the CM (scores and bands of
 * every state, flags): a CM reconfigured in place maps to a new upload. */
static uint64_t cm_signature(const CM_t *cm, int tr)
{
  uint64_t h = 1469598103934665603ULL;
  int v;
  h = fnv(h, &cm->M, sizeof(int)); h = fnv(h, &cm->W, sizeof(int));
  h = fnv(h, &cm->flags, sizeof(int)); h = fnv(h, &cm->search_opts, sizeof(int));
  h = fnv(h, &cm->el_selfsc, sizeof(float)); h = fnv(h, &cm->iel_selfsc, sizeof(int));
  h = fnv(h, cm->endsc, sizeof(float) * cm->M); h = fnv(h, cm->beginsc, sizeof(float) * cm->M);
  h = fnv(h, cm->iendsc, sizeof(int) * cm->M); h = fnv(h, cm->ibeginsc, sizeof(int) * cm->M);
  for (v = 0; v < cm->M; v++) {
    h = fnv(h, cm->tsc[v], sizeof(float) * MAXCONNECT);
    h = fnv(h, cm->itsc[v], sizeof(int) * MAXCONNECT);
    h = fnv(h, cm->oesc[v], sizeof(float) * (cm->sttype[v] == MP_st ? cm->abc->Kp * cm->abc->Kp : cm->abc->Kp));
  }
  if (cm->qdbinfo) {
    h = fnv(h, cm->qdbinfo->dmin1, sizeof(int) * cm->M); h = fnv(h, cm->qdbinfo->dmax1, sizeof(int) * cm->M);
    h = fnv(h, cm->qdbinfo->dmin2, sizeof(int) * cm->M); h = fnv(h, cm->qdbinfo->dmax2, sizeof(int) * cm->M);
  }
  h = fnv(h, &tr, sizeof(int));
  return h;
}

static int thread_state(adapter_thread_t **ret, char *errbuf)
{
  if (tls == NULL) {
    adapter_thread_t *t = calloc(1, sizeof(adapter_thread_t));
    const char *dev = getenv("INFERNAL_GB300_DEVICE");
    int status;
    if (t == NULL) ESL_FAIL(eslEMEM, errbuf, "Memory allocation error.\n");
    cmgb_logsum_init();
    if ((status = cmgb_ctx_create(dev ? atoi(dev) : 0, &t->ctx, errbuf)) != CMGB_OK) { free(t); return status; }
    t->hl = cmgb_hitlist_create();
    tls = t;
  }
  *ret = tls;
  return eslOK;
}

/* Flattens a configured CM into the library's model description and uploads
 * it; tr adds the truncated scanners' tables. */
static int upload_model(cmgb_ctx *ctx, const CM_t *cm, int tr, cmgb_model **ret, char *errbuf)
{
  const int M = cm->M, Kp = cm->abc->Kp, KK = Kp * Kp;
  cmgb_model_desc d;
  int v, x, p, status = eslEMEM;
  int8_t *sttype = NULL, *stid = NULL, *ndtype = NULL;
  float *tsc = NULL, *oesc = NULL, *lmesc = NULL, *rmesc = NULL, *g = NULL, *l = NULL;
  int *itsc = NULL, *ioesc = NULL, *ilmesc = NULL, *irmesc = NULL, *ig = NULL, *il = NULL;

  memset(&d, 0, sizeof(d));
  d.M = M; d.W = cm->W; d.K = cm->abc->K; d.Kp = Kp;
  d.flags = ((cm->flags & CMH_LOCAL_BEGIN) ? CMGB_LOCAL_BEGIN : 0) | ((cm->flags & CMH_LOCAL_END) ? CMGB_LOCAL_END : 0) |
            ((cm->search_opts & CM_SEARCH_CMNOTGREEDY) ? CMGB_NOTGREEDY : 0);
  if ((sttype = malloc(M)) == NULL || (stid = malloc(M)) == NULL) goto done;
  if ((tsc = calloc((size_t) M * 6, sizeof(float))) == NULL || (itsc = calloc((size_t) M * 6, sizeof(int))) == NULL) goto done;
  if ((oesc = calloc((size_t) M * KK, sizeof(float))) == NULL || (ioesc = calloc((size_t) M * KK, sizeof(int))) == NULL) goto done;
  for (v = 0; v < M; v++) {
    const int n = (cm->sttype[v] == MP_st) ? KK : (cm->sttype[v] == E_st || cm->sttype[v] == B_st ||
                                                    cm->sttype[v] == S_st || cm->sttype[v] == D_st) ? 0 : Kp;
    sttype[v] = (int8_t) cm->sttype[v]; stid[v] = (int8_t) cm->stid[v];
    for (x = 0; x < MAXCONNECT && x < 6; x++) { tsc[v * 6 + x] = cm->tsc[v][x]; itsc[v * 6 + x] = cm->itsc[v][x]; }
    for (x = 0; x < n; x++) { oesc[(size_t) v * KK + x] = cm->oesc[v][x]; ioesc[(size_t) v * KK + x] = cm->ioesc[v][x]; }
  }
  d.sttype = sttype; d.stid = stid; d.cfirst = cm->cfirst; d.cnum = cm->cnum;
  if (cm->qdbinfo) {
    d.dmin1 = cm->qdbinfo->dmin1; d.dmax1 = cm->qdbinfo->dmax1;
    d.dmin2 = cm->qdbinfo->dmin2; d.dmax2 = cm->qdbinfo->dmax2;
  }
  d.tsc = tsc; d.oesc = oesc; d.endsc = cm->endsc; d.beginsc = cm->beginsc; d.el_selfsc = cm->el_selfsc;
  d.itsc = itsc; d.ioesc = ioesc; d.iendsc = cm->iendsc; d.ibeginsc = cm->ibeginsc; d.iel_selfsc = cm->iel_selfsc;
  d.null = cm->null; d.null3_omega = cm->null3_omega;
  if (tr) {
    if (cm->trp == NULL || cm->lmesc == NULL || cm->rmesc == NULL || cm->emap == NULL) {
      status = eslEINCOMPAT;
      if (errbuf) snprintf(errbuf, eslERRBUFSIZE, "truncated scan: the CM has no truncation penalties, marginal scores or emit map\n");
      goto done;
    }
    if ((lmesc = malloc(sizeof(float) * M * Kp)) == NULL || (rmesc = malloc(sizeof(float) * M * Kp)) == NULL ||
        (ilmesc = malloc(sizeof(int) * M * Kp)) == NULL || (irmesc = malloc(sizeof(int) * M * Kp)) == NULL) goto done;
    if ((g = malloc(sizeof(float) * 3 * M)) == NULL || (l = malloc(sizeof(float) * 3 * M)) == NULL ||
        (ig = malloc(sizeof(int) * 3 * M)) == NULL || (il = malloc(sizeof(int) * 3 * M)) == NULL) goto done;
    if ((ndtype = malloc(cm->nodes)) == NULL) goto done;
    for (v = 0; v < M; v++)
      for (x = 0; x < Kp; x++) {
        lmesc[v * Kp + x] = cm->lmesc[v][x]; rmesc[v * Kp + x] = cm->rmesc[v][x];
        ilmesc[v * Kp + x] = cm->ilmesc[v][x]; irmesc[v * Kp + x] = cm->irmesc[v][x];
      }
    for (p = 0; p < 3; p++)
      for (v = 0; v < M; v++) {
        g[p * M + v] = cm->trp->g_ptyAA[p][v];  l[p * M + v] = cm->trp->l_ptyAA[p][v];
        ig[p * M + v] = cm->trp->ig_ptyAA[p][v]; il[p * M + v] = cm->trp->il_ptyAA[p][v];
      }
    for (x = 0; x < cm->nodes; x++) ndtype[x] = (int8_t) cm->ndtype[x];
    d.lmesc = lmesc; d.rmesc = rmesc; d.ilmesc = ilmesc; d.irmesc = irmesc;
    d.tr_g_pty = g; d.tr_l_pty = l; d.tr_ig_pty = ig; d.tr_il_pty = il;
    d.ndidx = cm->ndidx; d.emap_lpos = cm->emap->lpos; d.emap_rpos = cm->emap->rpos;
    d.clen = cm->clen; d.ndtype = ndtype; d.nodes = cm->nodes;
  }
  status = cmgb_model_create(ctx, &d, ret, errbuf);
 done:
  if (status == eslEMEM && errbuf) snprintf(errbuf, eslERRBUFSIZE, "Memory allocation error.\n");
  free(sttype); free(stid); free(tsc); free(itsc); free(oesc); free(ioesc);
  free(lmesc); free(rmesc); free(ilmesc); free(irmesc); free(g); free(l); free(ig); free(il); free(ndtype);
  return status;
}

static int get_model(adapter_thread_t *t, const CM_t *cm, int tr, cmgb_model **ret, char *errbuf)
{
  const uint64_t sig = cm_signature(cm, tr);
  int k, status;
  for (k = 0; k < ADAPTER_MODELS; k++)
    if (t->models[k].model && t->models[k].cm == cm && t->models[k].sig == sig && t->models[k].tr == tr) {
      *ret = t->models[k].model;
      return eslOK;
    }
  k = t->next; t->next = (t->next + 1) % ADAPTER_MODELS;
  if (t->models[k].model) { cmgb_model_destroy(t->models[k].model); t->models[k].model = NULL; }
  if ((status = upload_model(t->ctx, cm, tr, &t->models[k].model, errbuf)) != eslOK) return status;
  t->models[k].cm = cm; t->models[k].sig = sig; t->models[k].tr = tr;
  *ret = t->models[k].model;
  return eslOK;
}

/* Appends the library's hits to the caller's CM_TOPHITS with the fields the
 * reference scanner sets (see the header comment). */
static int copy_hits(const CM_t *cm, cmgb_hitlist *hl, CM_TOPHITS *hitlist, int64_t j0, char *errbuf)
{
  const int greedy = !(cm->search_opts & CM_SEARCH_CMNOTGREEDY);
  const int64_t n = cmgb_hitlist_count(hl);
  int64_t h;
  for (h = 0; h < n; h++) {
    cmgb_hit g;
    CM_HIT *hit = NULL;
    cmgb_hitlist_get(hl, h, &g);
    if (cm_tophits_CreateNextHit(hitlist, &hit) != eslOK) ESL_FAIL(eslEMEM, errbuf, "problem copying hit to hitlist, out of memory?");
    hit->start   = g.start;
    hit->stop    = g.stop;
    hit->root    = g.root;
    hit->mode    = (char) g.mode;
    hit->score   = g.score;
    hit->hmmonly = FALSE;
    if (greedy) hit->srcL = j0;
  }
  return eslOK;
}

typedef int (*std_scan_fn)(cmgb_ctx *, cmgb_model *, char *, int, const uint8_t *, int64_t, int64_t, float, cmgb_hitlist *,
                           int, float, int64_t *, int64_t *, float *, float *);

static int std_scan(const char *name, int want_inside, int ints_check, std_scan_fn fn, CM_t *cm, char *errbuf,
                    CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff, CM_TOPHITS *hitlist,
                    int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc, float *ret_sc)
{
  adapter_thread_t *t;
  cmgb_model *model;
  float *vsc = NULL, sc;
  int64_t envi, envj;
  int status;

  /* the reference's contract (src/cm_dpsearch.c:129-154, 1147-1171, 1774-1797) */
  if (!(cm->flags & CMH_BITS))         ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CMH_BITS flag is not raised.\n", name);
  if (j0 < i0)                         ESL_FAIL(eslEINCOMPAT, errbuf, "%s, i0: %" PRId64 " j0: %" PRId64 "d\n", name, i0, j0);
  if (dsq == NULL)                     ESL_FAIL(eslEINCOMPAT, errbuf, "%s, dsq is NULL\n", name);
  if (want_inside && !(cm->search_opts & CM_SEARCH_INSIDE)) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CM_SEARCH_INSIDE flag not raised", name);
  if (!want_inside && (cm->search_opts & CM_SEARCH_INSIDE)) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CM_SEARCH_INSIDE flag raised", name);
  if (smx == NULL)                     ESL_FAIL(eslEINCOMPAT, errbuf, "%s, smx == NULL\n", name);
  if (ints_check && !smx->ints_valid)  ESL_FAIL(eslEINCOMPAT, errbuf, "%s, smx->ints_valid if FALSE", name);
  if (!ints_check && !smx->floats_valid) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, smx->floats_valid if FALSE", name);
  if (cm->qdbinfo == NULL)             ESL_FAIL(eslEINCOMPAT, errbuf, "%s, cm->qdbinfo == NULL\n", name);
  if (qdbidx != SMX_NOQDB && qdbidx != SMX_QDB1_TIGHT && qdbidx != SMX_QDB2_LOOSE)
    ESL_FAIL(eslEINCOMPAT, errbuf, "%s, qdbidx is invalid", name);

  if ((status = thread_state(&t, errbuf)) != eslOK) return status;
  if ((status = get_model(t, cm, FALSE, &model, errbuf)) != eslOK) return status;
  if (ret_vsc != NULL && (vsc = malloc(sizeof(float) * cm->M)) == NULL) ESL_FAIL(eslEMEM, errbuf, "Memory allocation error.\n");
  cmgb_hitlist_clear(t->hl);
  status = fn(t->ctx, model, errbuf, qdbidx, dsq, i0, j0, cutoff, hitlist ? t->hl : NULL, do_null3, env_cutoff,
              &envi, &envj, vsc, &sc);
  if (status == CMGB_OK && hitlist != NULL) status = copy_hits(cm, t->hl, hitlist, j0, errbuf);
  if (status != CMGB_OK) { free(vsc); return status; }
  if (ret_envi) *ret_envi = envi;
  if (ret_envj) *ret_envj = envj;
  if (ret_vsc) *ret_vsc = vsc;
  if (ret_sc) *ret_sc = sc;
  return eslOK;
}

int FastCYKScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
                CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
                float *ret_sc)
{
  return std_scan("FastCYKScan", FALSE, FALSE, cmgb_FastCYKScan, cm, errbuf, smx, qdbidx, dsq, i0, j0, cutoff, hitlist,
                  do_null3, env_cutoff, ret_envi, ret_envj, ret_vsc, ret_sc);
}

int FastIInsideScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
                    CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
                    float *ret_sc)
{
  return std_scan("FastIInsideScan", TRUE, TRUE, cmgb_FastIInsideScan, cm, errbuf, smx, qdbidx, dsq, i0, j0, cutoff, hitlist,
                  do_null3, env_cutoff, ret_envi, ret_envj, ret_vsc, ret_sc);
}

/* the reference checks ints_valid here too (src/cm_dpsearch.c:1790) */
int FastFInsideScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
                    CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
                    float *ret_sc)
{
  return std_scan("FastFInsideScan", TRUE, TRUE, cmgb_FastFInsideScan, cm, errbuf, smx, qdbidx, dsq, i0, j0, cutoff, hitlist,
                  do_null3, env_cutoff, ret_envi, ret_envj, ret_vsc, ret_sc);
}

typedef int (*tr_scan_fn)(cmgb_ctx *, cmgb_model *, char *, int, int, const uint8_t *, int64_t, int64_t, float, cmgb_hitlist *,
                          int, float, int64_t *, int64_t *, float *, int *, float *);

static int tr_scan(const char *name, int want_inside, tr_scan_fn fn, CM_t *cm, char *errbuf, CM_TR_SCAN_MX *trsmx, int qdbidx,
                   int pass_idx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff, CM_TOPHITS *hitlist, int do_null3,
                   float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc, char *ret_mode, float *ret_sc)
{
  adapter_thread_t *t;
  cmgb_model *model;
  float *vsc = NULL, sc;
  int64_t envi, envj;
  int mode, status;

  /* the reference's contract (src/cm_dpsearch_trunc.c:131-136, 789-794) */
  if (!(cm->flags & CMH_BITS))         ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CMH_BITS flag is not raised.\n", name);
  if (j0 < i0)                         ESL_FAIL(eslEINCOMPAT, errbuf, "%s, i0: %" PRId64 " j0: %" PRId64 "d\n", name, i0, j0);
  if (dsq == NULL)                     ESL_FAIL(eslEINCOMPAT, errbuf, "%s, dsq is NULL\n", name);
  if (want_inside && !(cm->search_opts & CM_SEARCH_INSIDE)) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CM_SEARCH_INSIDE flag not raised", name);
  if (!want_inside && (cm->search_opts & CM_SEARCH_INSIDE)) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, CM_SEARCH_INSIDE flag raised", name);
  if (trsmx == NULL)                   ESL_FAIL(eslEINCOMPAT, errbuf, "%s, trsmx == NULL\n", name);
  if (want_inside && !trsmx->ints_valid)    ESL_FAIL(eslEINCOMPAT, errbuf, "%s, trsmx->ints_valid if FALSE", name);
  if (!want_inside && !trsmx->floats_valid) ESL_FAIL(eslEINCOMPAT, errbuf, "%s, trsmx->floats_valid if FALSE", name);

  if ((status = thread_state(&t, errbuf)) != eslOK) return status;
  if ((status = get_model(t, cm, TRUE, &model, errbuf)) != eslOK) return status;
  if (ret_vsc != NULL && (vsc = malloc(sizeof(float) * cm->M)) == NULL) ESL_FAIL(eslEMEM, errbuf, "Memory allocation error.\n");
  cmgb_hitlist_clear(t->hl);
  status = fn(t->ctx, model, errbuf, qdbidx, pass_idx, dsq, i0, j0, cutoff, hitlist ? t->hl : NULL, do_null3, env_cutoff,
              &envi, &envj, vsc, &mode, &sc);
  if (status == CMGB_OK && hitlist != NULL) status = copy_hits(cm, t->hl, hitlist, j0, errbuf);
  if (status != CMGB_OK) { free(vsc); return status; }
  if (ret_envi) *ret_envi = envi;
  if (ret_envj) *ret_envj = envj;
  if (ret_vsc) *ret_vsc = vsc;
  if (ret_mode) *ret_mode = (char) mode;
  if (ret_sc) *ret_sc = sc;
  return eslOK;
}

int RefTrCYKScan(CM_t *cm, char *errbuf, CM_TR_SCAN_MX *trsmx, int qdbidx, int pass_idx, ESL_DSQ *dsq, int64_t i0, int64_t j0,
                 float cutoff, CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj,
                 float **ret_vsc, char *ret_mode, float *ret_sc)
{
  return tr_scan("RefTrCYKScan", FALSE, cmgb_RefTrCYKScan, cm, errbuf, trsmx, qdbidx, pass_idx, dsq, i0, j0, cutoff, hitlist,
                 do_null3, env_cutoff, ret_envi, ret_envj, ret_vsc, ret_mode, ret_sc);
}

int RefITrInsideScan(CM_t *cm, char *errbuf, CM_TR_SCAN_MX *trsmx, int qdbidx, int pass_idx, ESL_DSQ *dsq, int64_t i0,
                     int64_t j0, float cutoff, CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi,
                     int64_t *ret_envj, float **ret_vsc, char *ret_mode, float *ret_sc)
{
  return tr_scan("RefITrInsideScan", TRUE, cmgb_RefITrInsideScan, cm, errbuf, trsmx, qdbidx, pass_idx, dsq, i0, j0, cutoff,
                 hitlist, do_null3, env_cutoff, ret_envi, ret_envj, ret_vsc, ret_mode, ret_sc);
}
