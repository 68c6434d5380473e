/* infernal_gb300.h -- C ABI of the GB300 query-dependent-banded (QDB) CM scanners.
 *
 * This library replaces the CPU scanning DP of Infernal's search pipeline:
 *
 *   FastCYKScan()      src/cm_dpsearch.c:90     (declared src/infernal.h:2710)
 *   FastIInsideScan()  src/cm_dpsearch.c:1106   (declared src/infernal.h:2712)
 *   FastFInsideScan()  src/cm_dpsearch.c:1731   (declared src/infernal.h:2713)
 *   RefTrCYKScan()     src/cm_dpsearch_trunc.c:79   (declared src/infernal.h:2722)
 *   RefITrInsideScan() src/cm_dpsearch_trunc.c:741  (declared src/infernal.h:2724)
 *
 * Every entry point keeps the reference scanner's argument meaning, return
 * codes and error text convention (status code + message in errbuf); the
 * only differences are that the model is passed as a flat, already
 * configured parameter block (cmgb_model_desc, uploaded once into a
 * cmgb_model) instead of a CM_t, the rolling scan matrix lives on the GPU
 * (cmgb_ctx) instead of a CM_SCAN_MX, and hits are appended to a
 * cmgb_hitlist instead of a CM_TOPHITS.  An Infernal build binds the
 * reference names to these calls with the adapter in
 * infernal_gb300/adapter/infernal_gb300_adapter.c, which defines
 * FastCYKScan() & co. with the reference prototypes and copies the CM_t
 * fields listed below.
 *
 * All pointers are plain host pointers, all sizes plain integers; nothing in
 * this header depends on CUDA, PyTorch or Easel headers.
 */
#ifndef INFERNAL_GB300_H
#define INFERNAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes: the Easel status codes the reference scanners return. */
#define CMGB_OK          0   /* eslOK        */
#define CMGB_EMEM        5   /* eslEMEM      */
#define CMGB_EINCOMPAT  10   /* eslEINCOMPAT */
#define CMGB_EINVAL     11   /* eslEINVAL    */
#define CMGB_ERANGE     16   /* eslERANGE    */
#define CMGB_ENODEV     30   /* no usable sm_103 GPU / CUDA runtime error */
#define CMGB_ERRBUFSIZE 128  /* eslERRBUFSIZE */

/* State types, unique state ids (src/infernal.h:193-243). */
#define CMGB_D_st   0
#define CMGB_MP_st  1
#define CMGB_ML_st  2
#define CMGB_MR_st  3
#define CMGB_IL_st  4
#define CMGB_IR_st  5
#define CMGB_S_st   6
#define CMGB_E_st   7
#define CMGB_B_st   8
#define CMGB_EL_st  9
#define CMGB_BEGL_S 3

/* Band sets (SMX_NOQDB / SMX_QDB1_TIGHT / SMX_QDB2_LOOSE, src/infernal.h). */
#define CMGB_NOQDB      0
#define CMGB_QDB1_TIGHT 1
#define CMGB_QDB2_LOOSE 2

/* Model flags (subset of cm->flags / cm->search_opts that the scanners read). */
#define CMGB_LOCAL_BEGIN  (1 << 0)   /* CMH_LOCAL_BEGIN */
#define CMGB_LOCAL_END    (1 << 1)   /* CMH_LOCAL_END   */
#define CMGB_NOTGREEDY    (1 << 2)   /* CM_SEARCH_CMNOTGREEDY: optimal (gamma) hit resolution */

/* Score sentinels (src/infernal.h:148-158). */
#define CMGB_IMPOSSIBLE (-1e36f)
#define CMGB_INFTY      987654321
#define CMGB_LOGSUM_TBL 23000

/* Pipeline pass indices (PLI_PASS_*, src/infernal.h:2097-2103); the
 * truncated scanners accept passes 2..5 (cm_TrFillFromPassIdx,
 * src/cm_dpsearch_trunc.c:3566). */
#define CMGB_PASS_STD_ANY         1
#define CMGB_PASS_5P_ONLY_FORCE   2
#define CMGB_PASS_3P_ONLY_FORCE   3
#define CMGB_PASS_5P_AND_3P_FORCE 4
#define CMGB_PASS_5P_AND_3P_ANY   5
#define CMGB_PASS_HMM_ONLY_ANY    6

/* Truncation modes of a hit (TRMODE_*, src/infernal.h). */
#define CMGB_TRMODE_J 3
#define CMGB_TRMODE_L 2
#define CMGB_TRMODE_R 1
#define CMGB_TRMODE_T 0
#define CMGB_TRMODE_UNKNOWN 4

/* Node types (src/infernal.h:209-216). */
#define CMGB_BIF_nd  0
#define CMGB_MATP_nd 1
#define CMGB_MATL_nd 2
#define CMGB_MATR_nd 3
#define CMGB_BEGL_nd 4
#define CMGB_BEGR_nd 5
#define CMGB_ROOT_nd 6
#define CMGB_END_nd  7
#define CMGB_END_E   18   /* unique state id of END_E: the state after a detached insert */

/* Flat view of a configured CM_t: exactly the fields the scanners read.
 * Per-state tables are indexed [v] for v in 0..M-1; tsc/itsc have a fixed
 * stride of 6 (MAXCONNECT) and oesc/ioesc a fixed stride of Kp*Kp (the
 * reference allocates Kp for singlet emitters and Kp*Kp for pair emitters;
 * only that prefix of each row is read). */
typedef struct {
  int          M;          /* cm->M */
  int          W;          /* cm->W, maximum hit length */
  int          K, Kp;      /* cm->abc->K, cm->abc->Kp (4 and 18 for RNA) */
  int          flags;      /* CMGB_LOCAL_BEGIN | CMGB_LOCAL_END | CMGB_NOTGREEDY */
  const int8_t *sttype;    /* cm->sttype[v] */
  const int8_t *stid;      /* cm->stid[v]   */
  const int   *cfirst;     /* cm->cfirst[v] */
  const int   *cnum;       /* cm->cnum[v]   */
  const int   *dmin1, *dmax1, *dmin2, *dmax2;  /* cm->qdbinfo bands; a band set may be NULL (both arrays):
                                                  scans then accept qdbidx 0 and the other set only */
  const float *tsc;        /* [M*6]     cm->tsc      */
  const float *oesc;       /* [M*Kp*Kp] cm->oesc     */
  const float *endsc;      /* [M]       cm->endsc    */
  const float *beginsc;    /* [M]       cm->beginsc  */
  float        el_selfsc;  /* cm->el_selfsc */
  const int   *itsc;       /* [M*6]     cm->itsc     */
  const int   *ioesc;      /* [M*Kp*Kp] cm->ioesc    */
  const int   *iendsc;     /* [M]       cm->iendsc   */
  const int   *ibeginsc;   /* [M]       cm->ibeginsc */
  int          iel_selfsc; /* cm->iel_selfsc */
  const float *null;       /* [K] cm->null, background for NULL3 */
  float        null3_omega;/* cm->null3_omega */
  /* Truncated scanning (cm->trp, cm->lmesc/rmesc, cm->emap); may be NULL
   * when the truncated scanners are not used. */
  const float *lmesc, *rmesc;     /* [M*Kp] marginal left/right emission scores */
  const int   *ilmesc, *irmesc;   /* [M*Kp] integer versions */
  const float *tr_g_pty;   /* [3*M] trp->g_ptyAA[pty_idx][v] (global begins) */
  const float *tr_l_pty;   /* [3*M] trp->l_ptyAA[pty_idx][v] (local begins)  */
  const int   *tr_ig_pty;  /* [3*M] trp->ig_ptyAA */
  const int   *tr_il_pty;  /* [3*M] trp->il_ptyAA */
  const int   *ndidx;      /* [M]     cm->ndidx[v] */
  const int   *emap_lpos;  /* [nodes] cm->emap->lpos */
  const int   *emap_rpos;  /* [nodes] cm->emap->rpos */
  int          clen;       /* cm->clen */
  const int8_t *ndtype;    /* [nodes] cm->ndtype[nd] (read by the truncated hit filter) */
  int          nodes;      /* cm->nodes */
} cmgb_model_desc;

/* One hit (the fields of CM_HIT that the scanners set, src/infernal.h:2424). */
typedef struct {
  int64_t start, stop;   /* 1-based sequence coordinates, start <= stop */
  int     root;          /* root state of the hit (0 or a local-begin state) */
  int     mode;          /* CMGB_TRMODE_* */
  float   score;         /* bit score (NULL3-corrected when requested) */
} cmgb_hit;

typedef struct cmgb_model_s   cmgb_model;
typedef struct cmgb_ctx_s     cmgb_ctx;
typedef struct cmgb_hitlist_s cmgb_hitlist;

/* ---- logsum tables (init_ilogsum / FLogsumInit, src/logsum.c:74, 138) ---- */
/* Fills the host copies once; must be called before the first scan. */
void cmgb_logsum_init(void);

/* ---- device contexts: per-thread scan matrix + stream (the GPU analogue of
 * the per-worker CM_SCAN_MX clone, src/cmsearch.c:2555) ---- */
int  cmgb_ctx_create(int device, cmgb_ctx **ret_ctx, char *errbuf);
void cmgb_ctx_destroy(cmgb_ctx *ctx);
/* Kernel launch shape override; 0 keeps the default of each field.
 * tile_rows: end positions per tile (the rolling-row depth, <= 128);
 * window_len: owned end positions per CTA work item; ctas_per_sm: resident
 * CTAs per SM (0: as many as fit); threads: threads per CTA (64..512);
 * arena: where the DP tiles live (0 automatic, 1 shared memory, 2 a per-CTA
 * global-memory arena served from L1/L2). */
int  cmgb_ctx_set_shape(cmgb_ctx *ctx, int tile_rows, int window_len, int ctas_per_sm, int threads, int arena);
/* Device time of the last scan's kernels in milliseconds (CUDA events). */
float cmgb_ctx_last_kernel_ms(const cmgb_ctx *ctx);
/* Number of this library's kernels launched by the last scan. */
int  cmgb_ctx_last_launches(const cmgb_ctx *ctx);
/* Host->device and device->host bytes the last scan moved. */
void cmgb_ctx_last_transfer_bytes(const cmgb_ctx *ctx, int64_t *h2d, int64_t *d2h);

/* ---- models: configured CM parameters uploaded to one device ---- */
int  cmgb_model_create(cmgb_ctx *ctx, const cmgb_model_desc *desc, cmgb_model **ret_model, char *errbuf);
void cmgb_model_destroy(cmgb_model *model);

/* Autotuner: times candidate shapes (tile rows = rolling-row depth, and
 * shared- vs global-memory tiles) for band set qdbidx and algo (0 CYK,
 * 1 integer Inside, 2 float Inside) on a seeded iid sample of sample_len residues (0: enough
 * windows of 8 W residues for two per resident CTA) and stores the fastest in the model; scans on a
 * context whose tile_rows is 0 use it.  Returns the choice when the
 * pointers are non-NULL. */
int  cmgb_autotune(cmgb_ctx *ctx, cmgb_model *model, int qdbidx, int algo, int64_t sample_len,
                   int *ret_tile_rows, int *ret_arena, char *errbuf);

/* ---- hit lists (the CM_TOPHITS subset the scanners append to) ---- */
cmgb_hitlist *cmgb_hitlist_create(void);
void     cmgb_hitlist_destroy(cmgb_hitlist *hl);
int64_t  cmgb_hitlist_count(const cmgb_hitlist *hl);
int      cmgb_hitlist_get(const cmgb_hitlist *hl, int64_t idx, cmgb_hit *ret_hit);
void     cmgb_hitlist_clear(cmgb_hitlist *hl);

/* ---- scanners ----
 * dsq is the Easel digitized sequence: dsq[1..L] residues (0..Kp-1), with
 * sentinels in dsq[0] and dsq[L+1]; only dsq[i0..j0] is read.
 * hitlist may be NULL (no hit reporting, as in the reference).
 * ret_vsc may be NULL; otherwise it must hold M floats and receives the best
 * score of every state (the reference allocates it for the caller; here the
 * caller owns it).  ret_envi/ret_envj/ret_sc may be NULL. */

/* Replaces FastCYKScan() (src/cm_dpsearch.c:90-681). */
int cmgb_FastCYKScan(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                     const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                     cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                     int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);

/* Replaces FastIInsideScan() (src/cm_dpsearch.c:1106-1693). */
int cmgb_FastIInsideScan(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                         const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                         cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                         int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);

/* Replaces FastFInsideScan() (src/cm_dpsearch.c:1731-2320): Inside over float
 * scores with the FLogsum table (src/logsum.c:160-168). */
int cmgb_FastFInsideScan(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                         const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                         cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                         int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);

/* Same scans with the residues already resident in device memory:
 * d_dsq points at a device copy of dsq[0..j0+1] (same indexing as dsq). */
int cmgb_FastCYKScan_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                         const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff,
                         cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                         int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);
int cmgb_FastIInsideScan_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                             const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff,
                             cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                             int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);
int cmgb_FastFInsideScan_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                             const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff,
                             cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                             int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc);

/* ---- truncated scanners ----
 * pass_idx is the pipeline pass (CMGB_PASS_5P_ONLY_FORCE, _3P_ONLY_FORCE,
 * _5P_AND_3P_FORCE or _5P_AND_3P_ANY); it selects the truncation modes that
 * are scored and the truncated-begin penalties (cm_TrFillFromPassIdx,
 * src/cm_dpsearch_trunc.c:3566), and which hits may be reported
 * (cm_hit_AllowTruncation, src/cm_tophits.c:3048); any other value returns
 * CMGB_EINVAL.  ret_mode (may be NULL) receives the mode (CMGB_TRMODE_*) of
 * the best-scoring parse; hits carry their own mode.  The model must have
 * been created with the truncation fields of cmgb_model_desc (lmesc ..
 * nodes); otherwise CMGB_EINCOMPAT.  Other arguments as for the standard
 * scanners; ret_vsc receives, as in the reference, the best score of each
 * state over all end positions for CYK and at the final end position j0 for
 * integer Inside. */

/* Replaces RefTrCYKScan() (src/cm_dpsearch_trunc.c:79-700, declared src/infernal.h:2722). */
int cmgb_RefTrCYKScan(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx, int pass_idx,
                      const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                      cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                      int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, int *ret_mode, float *ret_sc);

/* Replaces RefITrInsideScan() (src/cm_dpsearch_trunc.c:741-1338, declared src/infernal.h:2724). */
int cmgb_RefITrInsideScan(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx, int pass_idx,
                          const uint8_t *dsq, int64_t i0, int64_t j0, float cutoff,
                          cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                          int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, int *ret_mode, float *ret_sc);

/* Same truncated scans with device-resident residues (as the _dev scanners above). */
int cmgb_RefTrCYKScan_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx, int pass_idx,
                          const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff,
                          cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                          int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, int *ret_mode, float *ret_sc);
int cmgb_RefITrInsideScan_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx, int pass_idx,
                              const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff,
                              cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                              int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, int *ret_mode, float *ret_sc);

/* ---- batched scans ----
 * Runs nseq independent scans of one model in one persistent launch: what
 * the reference's callers do in a loop (pli_dispatch_cm_search per window,
 * src/cm_pipeline.c:4187; cmcalibrate per sequence, src/cmcalibrate.c:2338)
 * with one CTA work item per sequence, longest sequence first.  It has no
 * reference counterpart of its own; each sequence's results equal those of
 * the single-sequence scanner named by algo on that sequence over [1, L].
 * Sequence q is the Easel digital sequence at seqs + offsets[q]: a sentinel,
 * lengths[q] residues, a sentinel, all within seqs[0 .. seqs_len-1].
 * Outputs per sequence (arrays of nseq, each may be NULL): ret_nhits (hits
 * it added to hitlist, which receives sequence 0's hits, then sequence 1's,
 * ..., each in the single scanner's order, with start/stop local to the
 * sequence), ret_envi/ret_envj (local, -1 if none), ret_sc (best score),
 * ret_mode (mode of the best parse; CMGB_TRMODE_J for the standard scans).
 * pass_idx is read by the truncated algorithms only.  Per-state scores
 * (ret_vsc) are not produced here. */
#define CMGB_ALGO_CYK       0   /* FastCYKScan      */
#define CMGB_ALGO_IINSIDE   1   /* FastIInsideScan  */
#define CMGB_ALGO_FINSIDE   2   /* FastFInsideScan  */
#define CMGB_ALGO_TRCYK     3   /* RefTrCYKScan     */
#define CMGB_ALGO_ITRINSIDE 4   /* RefITrInsideScan */
int cmgb_ScanBatch(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int algo, int qdbidx, int pass_idx,
                   const uint8_t *seqs, int64_t seqs_len, const int64_t *offsets, const int64_t *lengths,
                   int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                   int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode);
/* The same with the residue buffer already in device memory (d_seqs, a
 * device address; no host->device copy of residues).  Sequences whose
 * candidate hits need NULL3 compositions are read back individually. */
int cmgb_ScanBatch_dev(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int algo, int qdbidx, int pass_idx,
                       const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets, const int64_t *lengths,
                       int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                       int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode);

/* ---- multi-model batched scans ----
 * Runs njobs (model, sequence) scans of several models in one persistent
 * launch (one launch per tile placement when the models' plans mix shared-
 * memory and global-memory arenas): what cmsearch / cmscan do when they
 * loop over models and sequences (src/cmscan.c, src/cmsearch.c: one
 * pli_dispatch_cm_search per model and window).  Job k scans sequence
 * job_seq[k] (laid out as in cmgb_ScanBatch) with models[job_model[k]] and
 * that model's cutoff cutoffs[job_model[k]]; (model, sequence) pairs must be
 * distinct, and the sequences of one model must not overlap in the buffer
 * (those of different models may).  Long sequences are cut into windows as in cmgb_ScanBatch, and
 * every window of every job enters one work queue, largest band area
 * (model cells per residue x window rows) first.  algo is one of the
 * standard scanners (CMGB_ALGO_CYK, _IINSIDE, _FINSIDE).  Each job's results
 * equal those of cmgb_ScanBatch with that model over that sequence.
 * Outputs per job (arrays of njobs, each may be NULL): ret_nhits (hits it
 * added to hitlist, which receives job 0's hits, then job 1's, ..., local
 * coordinates), ret_envi/ret_envj (local, -1 if none), ret_sc (best score).
 * All models must belong to ctx. */
int cmgb_ScanMulti(cmgb_ctx *ctx, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                   int algo, int qdbidx, const uint8_t *seqs, int64_t seqs_len, const int64_t *offsets,
                   const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                   cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                   int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc);
/* The same with the residue buffer already in device memory (d_seqs, a
 * device address); sequences whose candidate hits need NULL3 compositions are
 * read back individually. */
int cmgb_ScanMulti_dev(cmgb_ctx *ctx, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                       int algo, int qdbidx, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                       const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                       cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                       int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc);

/* ---- E-value calibration ----
 * cmcalibrate's exponential tail fit for one search mode of a configured
 * model (src/cmcalibrate.c: process_search_workunit :2328 scans random
 * sequence with FastCYKScan / FastIInsideScan at the QDB2 bands, NULL3 on;
 * fit_histogram :1930 fits the top hits with esl_exp_FitComplete).  Scans
 * total_len residues of seeded random sequence (pieces of seq_len residues
 * of a background whose GC content changes between segments) in one batched
 * launch with algo (CMGB_ALGO_CYK or CMGB_ALGO_IINSIDE), keeps the best
 * tail_per_mb hits per Mb (the reference's --ltailn 750 for local modes,
 * --gtailn 250 for glocal) and fits them by maximum likelihood: mu = the
 * lowest tail score, lambda = 1 / mean excess over mu.  The result fills the
 * fields of the CM file's ECM lines (cm_file.c: "ECMLC lambda mu_extrap
 * mu_orig dbsize nrandhits tailp").  Only the tail is collected, so
 * nrandhits = tail size and tailp = 1; E-values, which depend on
 * nrandhits * tailp only (E = Z / dbsize * nrandhits * tailp *
 * exp(-lambda (S - mu_orig))), are those of the reference's fit.  ret_ms:
 * scan kernel time. */
typedef struct {
  double  lambda, mu_extrap, mu_orig, dbsize;
  int64_t nrandhits;
  double  tailp;
} cmgb_expinfo;
int cmgb_Calibrate(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int algo, int64_t total_len, int64_t seq_len,
                   uint64_t seed, int tail_per_mb, cmgb_expinfo *ret, float *ret_ms);

/* ---- learned window pre-filter ----
 * No reference counterpart: a learned screen placed before the CYK stage.
 * Windows of 2W residues at stride W over [i0, j0] (window k starts at
 * i0 + kW, so every hit of length <= W lies inside the window where it
 * starts in the first half) are scored by a dilated 1-D convolution network
 * (one-hot ACGU; six convolutions of kernel 9, dilations 1..32, 4 -> 128 ->
 * 128 channels, ReLU; max over positions; linear read-out), BF16 weights and
 * activations, FP32 accumulation, on the tensor cores.  Weights: w0
 * [9 taps][4][128] f32 (first layer), w [5][9][128 out][128 in] BF16 bit
 * patterns (layers 2-6), bias [6][128] f32, wout [129] f32 (read-out
 * weights then bias).  cmgb_filter_windows takes residues in device memory
 * (indexed like dsq) and writes one logit per window to ret_logits (host,
 * max_windows entries); *ret_ms receives the device time. */
typedef struct cmgb_filter_s cmgb_filter;
int  cmgb_filter_create(cmgb_ctx *ctx, int W, const float *w0, const uint16_t *w, const float *bias,
                        const float *wout, cmgb_filter **ret_filter, char *errbuf);
void cmgb_filter_destroy(cmgb_filter *filter);
int  cmgb_filter_windows(cmgb_ctx *ctx, cmgb_filter *filter, const uint8_t *d_dsq, int64_t i0, int64_t j0,
                         float *ret_logits, int64_t max_windows, int64_t *ret_nwin, float *ret_ms, char *errbuf);
/* One network for several CMs: the convolutions are shared, every CM has its
 * own read-out (head).  wout holds nheads rows of 128 weights + bias;
 * cmgb_filter_windows then writes nheads logits per window (window-major:
 * ret_logits[win * nheads + h], room for max_windows * nheads floats).
 * cmgb_filter_create is the one-head case. */
#define CMGB_FILTER_MAX_HEADS 64
int  cmgb_filter_create_heads(cmgb_ctx *ctx, int W, int nheads, const float *w0, const uint16_t *w, const float *bias,
                              const float *wout, cmgb_filter **ret_filter, char *errbuf);

/* Training of the same network without batch normalisation (convolution,
 * bias, ReLU; the result loads into cmgb_filter_create as is), all on the
 * device: forward on the tensor cores keeping every activation; backward with
 * the input gradients on the tensor cores (BF16) and the weight gradients in
 * fp32; AdamW on fp32 master weights.  A trainer holds one batch size.
 * cmgb_filter_trainer_step takes host windows ([batch][2W] residue codes;
 * codes above 3 read as missing) and labels ([batch] 0/1); the loss is the
 * mean over the batch of -w y log s(z) - (1 - y) log(1 - s(z)), s the
 * logistic function, w = pos_weight; lr = 0 computes gradients without an
 * update.  _set / _get move the fp32 weights (w as [5][9][128][128] floats)
 * and, in _get, the last step's gradients (NULL pointers are skipped). */
typedef struct cmgb_filter_trainer_s cmgb_filter_trainer;
int  cmgb_filter_trainer_create(cmgb_ctx *ctx, int W, int batch, uint64_t seed, cmgb_filter_trainer **ret, char *errbuf);
void cmgb_filter_trainer_destroy(cmgb_filter_trainer *trainer);
int  cmgb_filter_trainer_set(cmgb_filter_trainer *trainer, const float *w0, const float *w, const float *bias,
                             const float *wout, char *errbuf);
int  cmgb_filter_trainer_step(cmgb_filter_trainer *trainer, const uint8_t *windows, const float *labels, float pos_weight,
                              float lr, float weight_decay, float *ret_loss, float *ret_ms, char *errbuf);
int  cmgb_filter_trainer_get(cmgb_filter_trainer *trainer, float *w0, float *w, float *bias, float *wout,
                             float *gw0, float *gw, float *gb, float *gwout, char *errbuf);
/* The several-head trainer: labels are [batch][nheads] (window-major), one
 * positive-class weight per head, the loss sums the heads' terms (each
 * averaged over the batch as above); wout / gwout hold nheads rows of 129.
 * cmgb_filter_trainer_create / _step are the one-head case. */
int  cmgb_filter_trainer_create_heads(cmgb_ctx *ctx, int W, int batch, int nheads, uint64_t seed,
                                      cmgb_filter_trainer **ret, char *errbuf);
int  cmgb_filter_trainer_step_heads(cmgb_filter_trainer *trainer, const uint8_t *windows, const float *labels,
                                    const float *pos_weights, float lr, float weight_decay, float *ret_loss, float *ret_ms,
                                    char *errbuf);

/* ---- allocation-free CYK scan ----
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc while they scan:
 *   - a host program whose own allocator (a deep-learning framework's caching
 *     allocator, a memory pool sized at start-up) owns the device memory, so
 *     that memory taken behind its back fragments or overruns its budget;
 *   - a long-running search service that allocates everything at start-up,
 *     because cudaMalloc can fail under memory pressure at run time and
 *     cudaMalloc/cudaFree synchronise the whole device, stalling the
 *     service's other streams in the middle of a query.
 * It runs the same CYK kernel as cmgb_FastCYKScan_dev, but the kernel's
 * scratch (per-CTA carry rows, bifurcation history rings, tile arena, work
 * counter and control block) lives in one static device array of
 * CMGB_NOALLOC_SCRATCH_BYTES (64 MiB) that every GPU loading this library
 * holds until the process exits; the call allocates nothing.  When a model
 * needs more scratch per CTA than fits, fewer CTAs run; if not even one CTA
 * fits, the call fails with CMGB_ERANGE.  The context's ctas_per_sm and
 * window_len settings are honoured within that limit.
 *
 * Set-up: the first call on a device, with that device current, looks up
 * the array's device address there (cudaGetSymbolAddress) and keeps it; make
 * that first call before any stream capture.  All calls share the array and
 * it keeps the last call's contents (each call clears what must start at
 * zero), so calls that overlap on the GPU (other host threads, other
 * streams, other contexts) race: serialise them.  The caller's current
 * device is restored before the call returns.
 *
 * The model's plan for qdbidx must already exist on this context (built by an
 * earlier cmgb_FastCYKScan / cmgb_FastCYKScan_dev / cmgb_autotune call);
 * otherwise the call returns CMGB_EINCOMPAT without building one.
 * Inputs: d_dsq as for cmgb_FastCYKScan_dev.  Outputs: the candidate cells
 * are written to the caller's device array d_cells[cell_cap] in no
 * particular order, their number to *ret_ncells: every root cell of [i0,j0]
 * whose CYK score is >= cutoff, or, for a model flagged CMGB_NOTGREEDY,
 * every cell whose score is > 0 (the candidates of optimal resolution) --
 * the same cells cmgb_FastCYKScan resolves its hit list from.  Envelope and
 * best score as in cmgb_FastCYKScan.  NULL3 and per-state scores are not
 * computed here.  The call waits for its kernel before it returns. */
#define CMGB_NOALLOC_SCRATCH_BYTES (64u << 20)
typedef struct {
  int64_t j;      /* end position of the cell */
  int     d;      /* its length: start = j - d + 1 */
  float   score;  /* CYK bit score of the root cell */
  int     root;   /* root state (0 or a local-begin state) */
  int     pad;
} cmgb_cell;
int cmgb_FastCYKScan_noalloc(cmgb_ctx *ctx, cmgb_model *model, char *errbuf, int qdbidx,
                             const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff, float env_cutoff,
                             cmgb_cell *d_cells, int cell_cap, int *ret_ncells,
                             int64_t *ret_envi, int64_t *ret_envj, float *ret_sc);

/* ---- measured issue peak (roofline denominator) ----
 * No reference counterpart: a diagnostic for the scan kernels' roofline.
 * Times 8 independent chains per thread of x = max(x + y, z) on every SM of
 * the context's device (2048 threads per SM; best of three timed launches,
 * CUDA events) and returns the arithmetic rate in operations per second,
 * counting the add and the max as one operation each: kind 0 fp32
 * (round-to-nearest add, the CYK fold), kind 1 int32 (the integer Inside's
 * add and combine, without its table lookup). */
int cmgb_measure_issue_peak(cmgb_ctx *ctx, int kind, double *ret_ops_per_s, char *errbuf);

/* DP cell count of one scan of [i0,j0] with band set qdbidx: the
 * algorithmic work unit, sum over j and non-E states of the band width
 * (the count cm_CountSearchDPCalcs() approximates, src/cm_dpsearch.c:3099). */
int64_t cmgb_count_cells(const cmgb_model_desc *desc, int qdbidx, int64_t L);

#ifdef __cplusplus
}
#endif
#endif /* INFERNAL_GB300_H */
