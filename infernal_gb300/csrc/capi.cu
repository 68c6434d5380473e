// capi.cu -- C ABI of the GB300 QDB scanners (declared in include/infernal_gb300.h).
//
// Device memory per context: the per-CTA carry rows and BEGL history rings
// (the scan matrix of src/cm_mx.c:5686, kept as rolling tiles), the residue
// staging buffer, the candidate-cell buffer and a small control block.
// Models hold the uploaded score tables and one execution plan per band set.
#ifdef CMGB_HOST_EMULATION
#include "cmgb_emu.h"
#endif
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <climits>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/infernal_gb300.h"
#include "hits.h"
#include "scan_kernel.cuh"
#include "scan_plan.h"
#include "trscan_kernel.cuh"

using namespace cmgb;

#define ERRF(code, ...) do { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, __VA_ARGS__); return (code); } while (0)
#define CUDA_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) ERRF(CMGB_ENODEV, "CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); } while (0)

#ifdef CMGB_HOST_EMULATION
static const int kDefaultThreads = CMGB_EMU_THREADS;
template <int ALG, bool GL, bool MULTI = false>
static void launch_qdb(int grid, int nt, size_t smem, cudaStream_t, const KParams &kp)
{
  std::vector<std::vector<float>> sm(grid, std::vector<float>(smem / 4 + 16));
  std::vector<EmuBarrier *> bars;
  std::vector<EmuWarp *> warps;
  for (int b = 0; b < grid; b++) bars.push_back(new EmuBarrier(nt));
  for (int b = 0; b < grid * (nt / 32); b++) warps.push_back(new EmuWarp);
  std::vector<std::thread> th;
  for (int b = 0; b < grid; b++)
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, b, t] {
        cmgb_emu_bar = bars[b]; cmgb_emu_warp = warps[b * (nt / 32) + t / 32]; cmgb_emu_lane = t & 31;
        qdb_scan_body<ALG, GL, MULTI>(kp, sm[b].data(), t, nt, b);
      });
  for (auto &x : th) x.join();
  for (auto *b : bars) delete b;
  for (auto *w : warps) delete w;
}
template <int ALG, bool GL>
static void launch_tr(int grid, int nt, size_t smem, cudaStream_t, const TrKParams &kp)
{
  std::vector<std::vector<float>> sm(grid, std::vector<float>(smem / 4 + 16));
  std::vector<EmuBarrier *> bars;
  std::vector<EmuWarp *> warps;
  for (int b = 0; b < grid; b++) bars.push_back(new EmuBarrier(nt));
  for (int b = 0; b < grid * (nt / 32); b++) warps.push_back(new EmuWarp);
  std::vector<std::thread> th;
  for (int b = 0; b < grid; b++)
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, b, t] {
        cmgb_emu_bar = bars[b]; cmgb_emu_warp = warps[b * (nt / 32) + t / 32]; cmgb_emu_lane = t & 31;
        tr_scan_body<ALG, GL>(kp, sm[b].data(), t, nt, b);
      });
  for (auto &x : th) x.join();
  for (auto *b : bars) delete b;
  for (auto *w : warps) delete w;
}
#else
static const int kDefaultThreads = 512;
template <int ALG, bool GL>
static void launch_tr(int grid, int nt, size_t smem, cudaStream_t s, const TrKParams &kp)
{
  tr_scan_kernel<ALG, GL><<<grid, nt, smem, s>>>(kp);
}
template <int ALG, bool GL>
static cudaError_t prepare_tr(int nt, int smem, int *blocks_per_sm)
{
  cudaError_t e = cudaFuncSetAttribute(tr_scan_kernel<ALG, GL>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, tr_scan_kernel<ALG, GL>, nt, smem);
}
template <int ALG, bool GL, bool MULTI = false>
static void launch_qdb(int grid, int nt, size_t smem, cudaStream_t s, const KParams &kp)
{
  qdb_scan_kernel<ALG, GL, MULTI><<<grid, nt, smem, s>>>(kp);
}
template <int ALG, bool GL, bool MULTI = false>
static cudaError_t prepare_qdb(int nt, int smem, int *blocks_per_sm)
{
  cudaError_t e = cudaFuncSetAttribute(qdb_scan_kernel<ALG, GL, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, qdb_scan_kernel<ALG, GL, MULTI>, nt, smem);
}
#endif
static const int kCandCap = 1 << 22;

// Runtime dispatch over (algorithm, tile placement, multi-model) to the kernel instantiations.
#ifndef CMGB_HOST_EMULATION
static cudaError_t prepare_any(int alg, bool gl, int nt, int smem, int *nb, bool multi = false)
{
  switch (alg * 4 + (gl ? 2 : 0) + (multi ? 1 : 0)) {
  case 0: return prepare_qdb<0, false, false>(nt, smem, nb);
  case 1: return prepare_qdb<0, false, true>(nt, smem, nb);
  case 2: return prepare_qdb<0, true, false>(nt, smem, nb);
  case 3: return prepare_qdb<0, true, true>(nt, smem, nb);
  case 4: return prepare_qdb<1, false, false>(nt, smem, nb);
  case 5: return prepare_qdb<1, false, true>(nt, smem, nb);
  case 6: return prepare_qdb<1, true, false>(nt, smem, nb);
  case 7: return prepare_qdb<1, true, true>(nt, smem, nb);
  case 8: return prepare_qdb<2, false, false>(nt, smem, nb);
  case 9: return prepare_qdb<2, false, true>(nt, smem, nb);
  case 10: return prepare_qdb<2, true, false>(nt, smem, nb);
  default: return prepare_qdb<2, true, true>(nt, smem, nb);
  }
}
#endif
static void launch_any(int alg, bool gl, int grid, int nt, size_t smem, cudaStream_t s, const KParams &kp, bool multi = false)
{
  switch (alg * 4 + (gl ? 2 : 0) + (multi ? 1 : 0)) {
  case 0: launch_qdb<0, false, false>(grid, nt, smem, s, kp); break;
  case 1: launch_qdb<0, false, true>(grid, nt, smem, s, kp); break;
  case 2: launch_qdb<0, true, false>(grid, nt, smem, s, kp); break;
  case 3: launch_qdb<0, true, true>(grid, nt, smem, s, kp); break;
  case 4: launch_qdb<1, false, false>(grid, nt, smem, s, kp); break;
  case 5: launch_qdb<1, false, true>(grid, nt, smem, s, kp); break;
  case 6: launch_qdb<1, true, false>(grid, nt, smem, s, kp); break;
  case 7: launch_qdb<1, true, true>(grid, nt, smem, s, kp); break;
  case 8: launch_qdb<2, false, false>(grid, nt, smem, s, kp); break;
  case 9: launch_qdb<2, false, true>(grid, nt, smem, s, kp); break;
  case 10: launch_qdb<2, true, false>(grid, nt, smem, s, kp); break;
  default: launch_qdb<2, true, true>(grid, nt, smem, s, kp); break;
  }
}

#ifndef CMGB_HOST_EMULATION
static cudaError_t prepare_tr_any(int alg, bool gl, int nt, int smem, int *nb)
{
  switch (alg * 2 + (gl ? 1 : 0)) {
  case 0: return prepare_tr<0, false>(nt, smem, nb);
  case 1: return prepare_tr<0, true>(nt, smem, nb);
  case 2: return prepare_tr<1, false>(nt, smem, nb);
  default: return prepare_tr<1, true>(nt, smem, nb);
  }
}
#endif
static void launch_tr_any(int alg, bool gl, int grid, int nt, size_t smem, cudaStream_t s, const TrKParams &kp)
{
  switch (alg * 2 + (gl ? 1 : 0)) {
  case 0: launch_tr<0, false>(grid, nt, smem, s, kp); break;
  case 1: launch_tr<0, true>(grid, nt, smem, s, kp); break;
  case 2: launch_tr<1, false>(grid, nt, smem, s, kp); break;
  default: launch_tr<1, true>(grid, nt, smem, s, kp); break;
  }
}

struct Control {            // device control block, zeroed/initialised per scan
  int queue;
  int ncand;
  int err;
  int pad;
  long long env[2];
  unsigned best;
  unsigned pad2[3];
};

struct cmgb_hitlist_s { std::vector<cmgb_hit> h; };

struct DevPlan {
  bool built = false;
  int T = 0, nt = 0, arena = -1;
  ScanPlan plan;
  StateInfo *d_states = nullptr;
  unsigned char *d_rec = nullptr;
};

struct DevTrPlan {
  bool built = false;
  int T = 0, nt = 0, arena = -1;
  ScanPlan plan;
  TrStateInfo *d_states = nullptr;
};

struct cmgb_model_s {
  cmgb_ctx *ctx = nullptr;
  int M = 0, W = 0, K = 0, Kp = 0, flags = 0;
  std::vector<float> null;
  float null3_omega = 0.f;
  // host copy of the description arrays (the plan builder re-reads them)
  std::vector<int8_t> sttype, stid;
  std::vector<int> cfirst, cnum, dmin1, dmax1, dmin2, dmax2, itsc, iendsc, ibeginsc;
  std::vector<float> tsc, endsc, beginsc, oesc;
  std::vector<int> ioesc;
  float el_selfsc = 0.f; int iel_selfsc = 0;
  cmgb_model_desc desc;      // points into the vectors above
  float *d_oesc = nullptr;
  int *d_ioesc = nullptr;
  DevPlan plans[3][3];       // [qdbidx][algorithm: 0 CYK, 1 integer Inside, 2 float Inside]
  // truncated scanning (present when the description carries the tables)
  bool has_tr = false;
  std::vector<float> lmesc, rmesc, tr_g, tr_l;
  std::vector<int> ilmesc, irmesc, tr_ig, tr_il, ndidx, emap_lpos, emap_rpos;
  std::vector<int8_t> ndtype;
  int clen = 0, nodes = 0;
  float *d_lmesc = nullptr, *d_rmesc = nullptr;
  int *d_ilmesc = nullptr, *d_irmesc = nullptr;
  DevTrPlan trplans[3][2];   // [qdbidx][0 TrCYK, 1 integer TrInside]
  int tuned_T[3][3] = {{0}}, tuned_arena[3][3] = {{0}};   // autotuner's choice (0: none yet)
};

struct cmgb_ctx_s {
  int device = 0;
  int nsm = 0;
  int max_smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  int last_launches = 0;
  int64_t last_h2d = 0, last_d2h = 0;
  int tile_rows = 0, window_len = 0, ctas_per_sm = 0, threads = kDefaultThreads, arena = 0;
  float *d_arena = nullptr; size_t arena_bytes = 0;
  // scratch
  float *d_carry = nullptr; size_t carry_bytes = 0;
  float *d_ring = nullptr; size_t ring_bytes = 0;
  unsigned char *d_dsq = nullptr; size_t dsq_bytes = 0;
  Cand *d_cand = nullptr; int cand_cap = 0;   // standard candidate buffer (grown by batched scans)
  Control *d_ctl = nullptr;
  unsigned *d_vsc = nullptr; int vsc_len = 0;
  int *d_ilog = nullptr;
  float *d_flog = nullptr;
  Control *h_ctl = nullptr;       // pinned
  std::vector<CandHost> h_cand;
  // truncated scans
  TrCand *d_trcand = nullptr; size_t trcand_bytes = 0;
  unsigned long long *d_winbest = nullptr; size_t winbest_bytes = 0;
  float *d_wmax = nullptr; size_t wmax_bytes = 0;
};

static int grow(void **p, size_t *cur, size_t need, char *errbuf)
{
  if (need <= *cur) return CMGB_OK;
  if (*p) cudaFree(*p);
  *p = nullptr; *cur = 0;
  size_t n = need + need / 4;
  if (cudaMalloc(p, n) != cudaSuccess) { *p = nullptr; ERRF(CMGB_EMEM, "out of device memory (%zu bytes)", n); }
  *cur = n;
  return CMGB_OK;
}

extern "C" void cmgb_logsum_init(void) { logsum_tables(nullptr, nullptr); }

extern "C" int cmgb_ctx_create(int device, cmgb_ctx **ret, char *errbuf)
{
  *ret = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device)
    ERRF(CMGB_ENODEV, "no CUDA device %d available", device);
  CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) ERRF(CMGB_ENODEV, "device %d is sm_%d%d; this library is built for sm_103a", device, prop.major, prop.minor);
  std::unique_ptr<cmgb_ctx> c(new cmgb_ctx);
  c->device = device;
  c->nsm = prop.multiProcessorCount;
  c->max_smem_optin = (int) prop.sharedMemPerBlockOptin;
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&c->ev0));
  CUDA_TRY(cudaEventCreate(&c->ev1));
  CUDA_TRY(cudaMalloc(&c->d_cand, sizeof(Cand) * (size_t) kCandCap));
  c->cand_cap = kCandCap;
  CUDA_TRY(cudaMalloc(&c->d_ctl, sizeof(Control)));
  CUDA_TRY(cudaMallocHost(&c->h_ctl, sizeof(Control)));
  const int *ilog;
  logsum_tables(nullptr, &ilog);
  CUDA_TRY(cudaMalloc(&c->d_ilog, sizeof(int) * 23000));
  CUDA_TRY(cudaMemcpy(c->d_ilog, ilog, sizeof(int) * 23000, cudaMemcpyHostToDevice));
  const float *flog;
  logsum_tables(&flog, nullptr);
  CUDA_TRY(cudaMalloc(&c->d_flog, sizeof(float) * 23000));
  CUDA_TRY(cudaMemcpy(c->d_flog, flog, sizeof(float) * 23000, cudaMemcpyHostToDevice));
  *ret = c.release();
  return CMGB_OK;
}

extern "C" void cmgb_ctx_destroy(cmgb_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  cudaFree(c->d_carry); cudaFree(c->d_ring); cudaFree(c->d_arena); cudaFree(c->d_dsq); cudaFree(c->d_cand);
  cudaFree(c->d_ctl); cudaFree(c->d_vsc); cudaFree(c->d_ilog); cudaFree(c->d_flog);
  cudaFree(c->d_trcand); cudaFree(c->d_winbest); cudaFree(c->d_wmax);
  cudaFreeHost(c->h_ctl);
  cudaEventDestroy(c->ev0); cudaEventDestroy(c->ev1);
  cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int cmgb_ctx_set_shape(cmgb_ctx *c, int tile_rows, int window_len, int ctas_per_sm, int threads, int arena)
{
  if (!c) return CMGB_EINVAL;
  if (arena < 0 || arena > 2) return CMGB_EINVAL;
  c->arena = arena;
  if (tile_rows < 0 || tile_rows > 128 || window_len < 0 || ctas_per_sm < 0 || ctas_per_sm > 8) return CMGB_EINVAL;
  if (threads != 0 && (threads < 64 || threads > 512 || threads % 32)) return CMGB_EINVAL;
  c->tile_rows = tile_rows;
  c->window_len = window_len;
  c->ctas_per_sm = ctas_per_sm;
#ifndef CMGB_HOST_EMULATION
  c->threads = threads ? threads : kDefaultThreads;
#endif
  return CMGB_OK;
}
extern "C" float cmgb_ctx_last_kernel_ms(const cmgb_ctx *c) { return c ? c->last_ms : 0.f; }
extern "C" int cmgb_ctx_last_launches(const cmgb_ctx *c) { return c ? c->last_launches : 0; }
extern "C" void cmgb_ctx_last_transfer_bytes(const cmgb_ctx *c, int64_t *h2d, int64_t *d2h)
{
  if (h2d) *h2d = c ? c->last_h2d : 0;
  if (d2h) *d2h = c ? c->last_d2h : 0;
}

extern "C" int cmgb_model_create(cmgb_ctx *c, const cmgb_model_desc *d, cmgb_model **ret, char *errbuf)
{
  *ret = nullptr;
  if (!c || !d) ERRF(CMGB_EINVAL, "cmgb_model_create: NULL argument");
  if (d->M < 2 || d->W < 1 || d->K != 4 || d->Kp != 18) ERRF(CMGB_EINCOMPAT, "cmgb_model_create: unsupported model shape (M=%d W=%d K=%d Kp=%d)", d->M, d->W, d->K, d->Kp);
  if (!d->sttype || !d->stid || !d->cfirst || !d->cnum || !d->tsc || !d->itsc || !d->oesc || !d->ioesc || !d->endsc ||
      !d->beginsc || !d->iendsc || !d->ibeginsc || !d->null)
    ERRF(CMGB_EINVAL, "cmgb_model_create: a required table of the model description is NULL");
  // band sets are optional (a model without query-dependent bands scans with qdbidx 0 only)
  if (!d->dmin1 != !d->dmax1 || !d->dmin2 != !d->dmax2)
    ERRF(CMGB_EINVAL, "cmgb_model_create: a band set needs both its dmin and its dmax array");
  const int M = d->M, KK = d->Kp * d->Kp;
  std::unique_ptr<cmgb_model> m(new cmgb_model);
  m->ctx = c; m->M = M; m->W = d->W; m->K = d->K; m->Kp = d->Kp; m->flags = d->flags;
  m->null.assign(d->null, d->null + d->K);
  m->null3_omega = d->null3_omega;
  m->sttype.assign(d->sttype, d->sttype + M); m->stid.assign(d->stid, d->stid + M);
  m->cfirst.assign(d->cfirst, d->cfirst + M); m->cnum.assign(d->cnum, d->cnum + M);
  if (d->dmin1) { m->dmin1.assign(d->dmin1, d->dmin1 + M); m->dmax1.assign(d->dmax1, d->dmax1 + M); }
  if (d->dmin2) { m->dmin2.assign(d->dmin2, d->dmin2 + M); m->dmax2.assign(d->dmax2, d->dmax2 + M); }
  m->tsc.assign(d->tsc, d->tsc + 6 * M); m->itsc.assign(d->itsc, d->itsc + 6 * M);
  m->endsc.assign(d->endsc, d->endsc + M); m->beginsc.assign(d->beginsc, d->beginsc + M);
  m->iendsc.assign(d->iendsc, d->iendsc + M); m->ibeginsc.assign(d->ibeginsc, d->ibeginsc + M);
  m->el_selfsc = d->el_selfsc == 0.0f ? 0.0f : d->el_selfsc; m->iel_selfsc = d->iel_selfsc;
  m->oesc.assign(d->oesc, d->oesc + (size_t) M * KK);
  m->ioesc.assign(d->ioesc, d->ioesc + (size_t) M * KK);
  // The CYK kernels take maxima with the max instruction, which orders -0.0
  // below +0.0 where ESL_MAX keeps its second operand; DP values can be -0.0
  // only through -0.0 table entries, so those (configured log2-odds tables
  // hold none) are stored as +0.0: the same values, and the kernels' maxima
  // then equal ESL_MAX bit for bit
  auto no_neg_zero = [](std::vector<float> &v) { for (float &x : v) if (x == 0.0f) x = 0.0f; };
  no_neg_zero(m->tsc); no_neg_zero(m->endsc); no_neg_zero(m->beginsc); no_neg_zero(m->oesc);
  const float el_sc = d->el_selfsc == 0.0f ? 0.0f : d->el_selfsc;
  std::memset(&m->desc, 0, sizeof(m->desc));
  cmgb_model_desc &D = m->desc;
  D.M = M; D.W = d->W; D.K = d->K; D.Kp = d->Kp; D.flags = d->flags;
  D.sttype = m->sttype.data(); D.stid = m->stid.data(); D.cfirst = m->cfirst.data(); D.cnum = m->cnum.data();
  D.dmin1 = m->dmin1.empty() ? nullptr : m->dmin1.data(); D.dmax1 = m->dmax1.empty() ? nullptr : m->dmax1.data();
  D.dmin2 = m->dmin2.empty() ? nullptr : m->dmin2.data(); D.dmax2 = m->dmax2.empty() ? nullptr : m->dmax2.data();
  D.tsc = m->tsc.data(); D.itsc = m->itsc.data(); D.endsc = m->endsc.data(); D.beginsc = m->beginsc.data();
  D.iendsc = m->iendsc.data(); D.ibeginsc = m->ibeginsc.data();
  D.el_selfsc = el_sc; D.iel_selfsc = d->iel_selfsc;
  D.null = m->null.data(); D.null3_omega = d->null3_omega;
  D.oesc = m->oesc.data(); D.ioesc = m->ioesc.data();
  if (cudaSetDevice(c->device) != cudaSuccess) ERRF(CMGB_ENODEV, "cudaSetDevice failed");
  if (cudaMalloc(&m->d_oesc, sizeof(float) * (size_t) M * KK) != cudaSuccess ||
      cudaMalloc(&m->d_ioesc, sizeof(int) * (size_t) M * KK) != cudaSuccess)
    ERRF(CMGB_EMEM, "out of device memory for emission tables");
  CUDA_TRY(cudaMemcpy(m->d_oesc, m->oesc.data(), sizeof(float) * (size_t) M * KK, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(m->d_ioesc, d->ioesc, sizeof(int) * (size_t) M * KK, cudaMemcpyHostToDevice));
  // truncated scanning tables (cm->lmesc/rmesc, cm->trp, cm->emap), when given
  if (d->lmesc && d->rmesc && d->ilmesc && d->irmesc && d->tr_g_pty && d->tr_l_pty && d->tr_ig_pty && d->tr_il_pty &&
      d->ndidx && d->emap_lpos && d->emap_rpos && d->ndtype && d->nodes > 0) {
    const size_t MK = (size_t) M * d->Kp;
    m->lmesc.assign(d->lmesc, d->lmesc + MK); m->rmesc.assign(d->rmesc, d->rmesc + MK);
    m->ilmesc.assign(d->ilmesc, d->ilmesc + MK); m->irmesc.assign(d->irmesc, d->irmesc + MK);
    m->tr_g.assign(d->tr_g_pty, d->tr_g_pty + 3 * M); m->tr_l.assign(d->tr_l_pty, d->tr_l_pty + 3 * M);
    no_neg_zero(m->lmesc); no_neg_zero(m->rmesc); no_neg_zero(m->tr_g); no_neg_zero(m->tr_l);
    m->tr_ig.assign(d->tr_ig_pty, d->tr_ig_pty + 3 * M); m->tr_il.assign(d->tr_il_pty, d->tr_il_pty + 3 * M);
    m->ndidx.assign(d->ndidx, d->ndidx + M);
    m->nodes = d->nodes; m->clen = d->clen;
    m->ndtype.assign(d->ndtype, d->ndtype + d->nodes);
    m->emap_lpos.assign(d->emap_lpos, d->emap_lpos + d->nodes); m->emap_rpos.assign(d->emap_rpos, d->emap_rpos + d->nodes);
    D.lmesc = m->lmesc.data(); D.rmesc = m->rmesc.data(); D.ilmesc = m->ilmesc.data(); D.irmesc = m->irmesc.data();
    D.tr_g_pty = m->tr_g.data(); D.tr_l_pty = m->tr_l.data(); D.tr_ig_pty = m->tr_ig.data(); D.tr_il_pty = m->tr_il.data();
    D.ndidx = m->ndidx.data(); D.ndtype = m->ndtype.data(); D.emap_lpos = m->emap_lpos.data(); D.emap_rpos = m->emap_rpos.data();
    D.clen = m->clen; D.nodes = m->nodes;
    if (cudaMalloc(&m->d_lmesc, sizeof(float) * MK) != cudaSuccess || cudaMalloc(&m->d_rmesc, sizeof(float) * MK) != cudaSuccess ||
        cudaMalloc(&m->d_ilmesc, sizeof(int) * MK) != cudaSuccess || cudaMalloc(&m->d_irmesc, sizeof(int) * MK) != cudaSuccess)
      ERRF(CMGB_EMEM, "out of device memory for marginal emission tables");
    CUDA_TRY(cudaMemcpy(m->d_lmesc, m->lmesc.data(), sizeof(float) * MK, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(m->d_rmesc, m->rmesc.data(), sizeof(float) * MK, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(m->d_ilmesc, d->ilmesc, sizeof(int) * MK, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(m->d_irmesc, d->irmesc, sizeof(int) * MK, cudaMemcpyHostToDevice));
    m->has_tr = true;
  }
  *ret = m.release();
  return CMGB_OK;
}

extern "C" void cmgb_model_destroy(cmgb_model *m)
{
  if (!m) return;
  cudaSetDevice(m->ctx->device);
  cudaFree(m->d_oesc); cudaFree(m->d_ioesc);
  cudaFree(m->d_lmesc); cudaFree(m->d_rmesc); cudaFree(m->d_ilmesc); cudaFree(m->d_irmesc);
  for (auto &row : m->plans) for (auto &p : row) { cudaFree(p.d_states); cudaFree(p.d_rec); }
  for (auto &row : m->trplans) for (auto &p : row) cudaFree(p.d_states);
  delete m;
}

extern "C" cmgb_hitlist *cmgb_hitlist_create(void) { return new cmgb_hitlist; }
extern "C" void cmgb_hitlist_destroy(cmgb_hitlist *hl) { delete hl; }
extern "C" int64_t cmgb_hitlist_count(const cmgb_hitlist *hl) { return hl ? (int64_t) hl->h.size() : 0; }
extern "C" int cmgb_hitlist_get(const cmgb_hitlist *hl, int64_t i, cmgb_hit *h)
{
  if (!hl || !h || i < 0 || i >= (int64_t) hl->h.size()) return CMGB_EINVAL;
  *h = hl->h[i];
  return CMGB_OK;
}
extern "C" void cmgb_hitlist_clear(cmgb_hitlist *hl) { if (hl) hl->h.clear(); }

// Builds (once) the plan of band set qdbidx for the context's tile size,
// shrinking the tile until its shared memory fits the device.
static int get_plan(cmgb_model *m, int qdbidx, int alg, DevPlan **ret, char *errbuf)
{
  cmgb_ctx *c = m->ctx;
  if ((qdbidx == 1 && m->dmin1.empty()) || (qdbidx == 2 && m->dmin2.empty()))
    ERRF(CMGB_EINCOMPAT, "the model was created without band set %d (qdbidx %d)", qdbidx, qdbidx);
  DevPlan &dp = m->plans[qdbidx][alg];
  // shape: the context's explicit choice, else the autotuner's, else 96 rows
  // (in global memory unless the context asks for shared)
  const int wantT = c->tile_rows ? c->tile_rows : (m->tuned_T[qdbidx][alg] ? m->tuned_T[qdbidx][alg] : 96);
  const int wantA = c->tile_rows ? c->arena : (m->tuned_T[qdbidx][alg] ? m->tuned_arena[qdbidx][alg] : c->arena);
  if (dp.built && dp.T == wantT && dp.nt == c->threads && dp.arena == wantA) { *ret = &dp; return CMGB_OK; }
  if (dp.d_states) { cudaFree(dp.d_states); dp.d_states = nullptr; }
  if (dp.d_rec) { cudaFree(dp.d_rec); dp.d_rec = nullptr; }
  PlanOut po;
  int T = wantT;
  for (;;) {
    po = PlanOut();
    // arena: 1 shared memory, 2 global memory, 0 shared when it fits the device, else global
    bool gl = wantA == 2;
    if (!build_plan(&m->desc, qdbidx, T, c->threads, alg == 1, gl, &po)) ERRF(CMGB_EINCOMPAT, "%s", po.err.c_str());
    if (!gl && wantA == 0 && po.plan.smem_bytes + 64 > c->max_smem_optin) {
      po = PlanOut();
      if (!build_plan(&m->desc, qdbidx, T, c->threads, alg == 1, true, &po)) ERRF(CMGB_EINCOMPAT, "%s", po.err.c_str());
    }
    if (po.plan.smem_bytes + 64 <= c->max_smem_optin) break;
    if (T <= 2) ERRF(CMGB_ERANGE, "model needs %d bytes of shared memory per CTA even with 2-row tiles", po.plan.smem_bytes);
    T = T > 8 ? T - 4 : T - 2;
  }
  build_records(&m->desc, alg == 1, &po);
  CUDA_TRY(cudaMalloc(&dp.d_rec, po.records.size()));
  CUDA_TRY(cudaMemcpy(dp.d_rec, po.records.data(), po.records.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMalloc(&dp.d_states, sizeof(StateInfo) * po.phases.size()));
  CUDA_TRY(cudaMemcpy(dp.d_states, po.phases.data(), sizeof(StateInfo) * po.phases.size(), cudaMemcpyHostToDevice));
  dp.plan = po.plan;
  dp.T = wantT;
  dp.nt = c->threads;
  dp.arena = wantA;
  dp.built = true;
  *ret = &dp;
  return CMGB_OK;
}

// Common driver of the standard scanners.  dev_dsq: device residues indexed
// by sequence coordinate (may be shifted); host_dsq: host residues (for
// NULL3), may be NULL when do_null3 is FALSE or the device copy suffices.
static int scan_std(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int alg,
                    const uint8_t *host_dsq, const uint8_t *dev_dsq_in, int64_t i0, int64_t j0,
                    float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                    int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, float *ret_sc)
{
  const char *fn = alg == 1 ? "FastIInsideScan" : alg == 2 ? "FastFInsideScan" : "FastCYKScan";
  if (!c || !m) ERRF(CMGB_EINVAL, "%s, NULL context or model", fn);
  if (j0 < i0) ERRF(CMGB_EINCOMPAT, "%s, i0: %lld j0: %lld", fn, (long long) i0, (long long) j0);
  if (i0 < 1) ERRF(CMGB_EINCOMPAT, "%s, i0 must be >= 1", fn);
  if (host_dsq == nullptr && dev_dsq_in == nullptr) ERRF(CMGB_EINCOMPAT, "%s, dsq is NULL", fn);
  if (qdbidx < 0 || qdbidx > 2) ERRF(CMGB_EINCOMPAT, "%s, qdbidx is invalid", fn);
  int st;
  CUDA_TRY(cudaSetDevice(c->device));
  DevPlan *dp;
  if ((st = get_plan(m, qdbidx, alg, &dp, errbuf)) != CMGB_OK) return st;
  const ScanPlan &P = dp->plan;
  const int64_t L = j0 - i0 + 1;
  const int W = m->W;

  // residues: device copy of dsq[lo .. j0+1]
  const unsigned char *d_dsq;
  int64_t lo = i0 - W - 1; if (lo < 0) lo = 0;
  if (dev_dsq_in) d_dsq = dev_dsq_in;
  else {
    size_t need = (size_t) (j0 + 2 - lo);
    if ((st = grow((void **) &c->d_dsq, &c->dsq_bytes, need, errbuf)) != CMGB_OK) return st;
    CUDA_TRY(cudaMemcpyAsync(c->d_dsq, host_dsq + lo, need, cudaMemcpyHostToDevice, c->stream));
    d_dsq = c->d_dsq - lo;
  }
  c->last_h2d = dev_dsq_in ? 0 : (int64_t) (j0 + 2 - lo);
  c->last_h2d += (int64_t) sizeof(Control);
  c->last_d2h = (int64_t) sizeof(Control) + (ret_vsc ? (int64_t) sizeof(unsigned) * m->M : 0);

  // launch shape
  const bool gl = P.arena_global != 0;
  int cps = c->ctas_per_sm;
  if (cps == 0) {
#ifndef CMGB_HOST_EMULATION
    int nb = 1;
    CUDA_TRY(prepare_any(alg, gl, c->threads, P.smem_bytes, &nb));
    cps = nb < 1 ? 1 : nb;
#else
    cps = 1;
#endif
  }
  int grid_max = c->nsm * cps;
  int64_t win = c->window_len;
  if (win <= 0) {
    win = (L + grid_max - 1) / grid_max;
    int64_t minwin = 8LL * W;
    if (win < minwin) win = minwin;
  }
  win = ((win + P.T - 1) / P.T) * P.T;
  int64_t nwin = (L + win - 1) / win;
  if (nwin > INT_MAX) ERRF(CMGB_ERANGE, "%s, too many windows", fn);
  int grid = (int) std::min<int64_t>(nwin, grid_max);

  size_t carry_need = sizeof(float) * 2 * (size_t) P.carry_elems * grid;
  size_t ring_need = sizeof(float) * (size_t) P.ring_elems * grid;
  if ((st = grow((void **) &c->d_carry, &c->carry_bytes, carry_need, errbuf)) != CMGB_OK) return st;
  if ((st = grow((void **) &c->d_ring, &c->ring_bytes, ring_need, errbuf)) != CMGB_OK) return st;
  if (gl && (st = grow((void **) &c->d_arena, &c->arena_bytes, sizeof(float) * (size_t) P.arena_elems * grid, errbuf)) != CMGB_OK) return st;
  if (ret_vsc && c->vsc_len < m->M) {
    cudaFree(c->d_vsc); c->d_vsc = nullptr;
    if (cudaMalloc(&c->d_vsc, sizeof(unsigned) * m->M) != cudaSuccess) ERRF(CMGB_EMEM, "out of device memory");
    c->vsc_len = m->M;
  }
  Control *h = c->h_ctl;
  std::memset(h, 0, sizeof(Control));
  h->env[0] = LLONG_MAX; h->env[1] = -1;
  CUDA_TRY(cudaMemcpyAsync(c->d_ctl, h, sizeof(Control), cudaMemcpyHostToDevice, c->stream));
  if (ret_vsc) CUDA_TRY(cudaMemsetAsync(c->d_vsc, 0, sizeof(unsigned) * m->M, c->stream));

  KParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.st = dp->d_states; kp.plan = P; kp.rec = dp->d_rec; kp.arena = c->d_arena;
  kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc; kp.ilog = c->d_ilog; kp.flog = c->d_flog;
  kp.dsq = d_dsq; kp.i0 = i0; kp.j0 = j0; kp.win_len = win; kp.nwin = (int) nwin;
  kp.queue = &c->d_ctl->queue; kp.carry = c->d_carry; kp.ring = c->d_ring;
  kp.cand = c->d_cand; kp.ncand = &c->d_ctl->ncand; kp.cand_cap = c->cand_cap;
  const bool greedy = !(m->flags & CMGB_NOTGREEDY);
  kp.cand_cut = cutoff; kp.cand_pos = (hitlist && !greedy) ? 1 : 0;
  if (!hitlist) { kp.cand_cut = 3.0e38f; kp.cand_pos = 0; }
  kp.env_cut = env_cutoff; kp.env = c->d_ctl->env;
  kp.vsc = ret_vsc ? c->d_vsc : nullptr; kp.best = &c->d_ctl->best; kp.err = &c->d_ctl->err;

  const size_t smem = (size_t) P.smem_bytes;
#ifndef CMGB_HOST_EMULATION
  {
    int nb_unused = 0;
    CUDA_TRY(prepare_any(alg, gl, c->threads, P.smem_bytes, &nb_unused));
  }
#endif
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  launch_any(alg, gl, grid, c->threads, smem, c->stream, kp);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  CUDA_TRY(cudaMemcpyAsync(h, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
  std::vector<unsigned> vscu;
  if (ret_vsc) { vscu.resize(m->M); CUDA_TRY(cudaMemcpyAsync(vscu.data(), c->d_vsc, sizeof(unsigned) * m->M, cudaMemcpyDeviceToHost, c->stream)); }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  c->last_launches = 1;
  if (h->err & 2) ERRF(CMGB_ENODEV, "%s, a bounded device wait ran out (phase record copy)", fn);
  if (h->err & 1) ERRF(CMGB_ERANGE, "%s, more than %d candidate hit cells; raise the cutoff", fn, c->cand_cap);

  auto u2f = [](unsigned u) { if (u == 0) return CMGB_IMPOSSIBLE; unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u; float f; std::memcpy(&f, &b, 4); return f; };
  const float best = u2f(h->best);
  if (ret_sc) *ret_sc = best;
  if (ret_envi) *ret_envi = (h->env[1] < 0) ? -1 : h->env[0];
  if (ret_envj) *ret_envj = (h->env[1] < 0) ? -1 : h->env[1];
  if (ret_vsc) { for (int v = 0; v < m->M; v++) ret_vsc[v] = u2f(vscu[v]); ret_vsc[0] = best; }

  if (hitlist) {
    const int n = h->ncand;
    c->h_cand.resize(n);
    if (n > 0) CUDA_TRY(cudaMemcpy(c->h_cand.data(), c->d_cand, sizeof(Cand) * n, cudaMemcpyDeviceToHost));
    c->last_d2h += (int64_t) sizeof(Cand) * n;
    std::vector<uint8_t> res_copy;
    const uint8_t *hd = host_dsq;
    if (do_null3 && n > 0 && hd == nullptr) {
      // device-resident residues: fetch [i0, j0] for the composition counts
      res_copy.resize((size_t) (j0 + 2));
      CUDA_TRY(cudaMemcpy(res_copy.data() + i0, dev_dsq_in + i0, (size_t) L, cudaMemcpyDeviceToHost));
      c->last_d2h += L;
      hd = res_copy.data();
    }
    ResolveArgs ra;
    ra.null = m->null.data(); ra.K = m->K; ra.null3_omega = m->null3_omega; ra.do_null3 = do_null3;
    ra.greedy = greedy ? 1 : 0; ra.cutoff = cutoff; ra.i0 = i0; ra.j0 = j0; ra.dsq = hd;
    resolve_hits(c->h_cand, ra, hitlist->h);
  }
  return CMGB_OK;
}

extern "C" int cmgb_FastCYKScan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *dsq, int64_t i0, int64_t j0,
                                float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                float *vsc, float *sc)
{
  if (dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastCYKScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 0, dsq, nullptr, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}
extern "C" int cmgb_FastIInsideScan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *dsq, int64_t i0, int64_t j0,
                                    float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                    float *vsc, float *sc)
{
  if (dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastIInsideScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 1, dsq, nullptr, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}
extern "C" int cmgb_FastCYKScan_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *d_dsq, int64_t i0, int64_t j0,
                                    float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                    float *vsc, float *sc)
{
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastCYKScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 0, nullptr, d_dsq, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}
extern "C" int cmgb_FastIInsideScan_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *d_dsq, int64_t i0, int64_t j0,
                                        float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                        float *vsc, float *sc)
{
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastIInsideScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 1, nullptr, d_dsq, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}

extern "C" int cmgb_FastFInsideScan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *dsq, int64_t i0, int64_t j0,
                                    float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                    float *vsc, float *sc)
{
  if (dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastFInsideScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 2, dsq, nullptr, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}
extern "C" int cmgb_FastFInsideScan_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, const uint8_t *d_dsq, int64_t i0, int64_t j0,
                                        float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff, int64_t *envi, int64_t *envj,
                                        float *vsc, float *sc)
{
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastFInsideScan, dsq is NULL");
  return scan_std(c, m, errbuf, qdbidx, 2, nullptr, d_dsq, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, sc);
}

// ---------------------------------------------------------------------------
// Truncated scanners (RefTrCYKScan / RefITrInsideScan).
static const int kTrCandCap = 1 << 21;          // initial truncated candidate capacity (grows on demand)
static const int64_t kTrCandMax = (int64_t) 1 << 27;

// Capacity of the context's truncated candidate buffer, grown to at least `need` entries.
static int tr_cand_reserve(cmgb_ctx *c, int64_t need, int *cap, char *errbuf)
{
  if (need > kTrCandMax) ERRF(CMGB_ERANGE, "more than %lld candidate root cells; raise the cutoff", (long long) kTrCandMax);
  int st = grow((void **) &c->d_trcand, &c->trcand_bytes, sizeof(TrCand) * (size_t) std::max<int64_t>(need, kTrCandCap), errbuf);
  if (st != CMGB_OK) return st;
  *cap = (int) std::min<int64_t>((int64_t) (c->trcand_bytes / sizeof(TrCand)), kTrCandMax);
  return CMGB_OK;
}

static int get_tr_plan(cmgb_model *m, int qdbidx, int alg, DevTrPlan **ret, char *errbuf)
{
  if ((qdbidx == 1 && m->dmin1.empty()) || (qdbidx == 2 && m->dmin2.empty()))
    ERRF(CMGB_EINCOMPAT, "the model was created without band set %d (qdbidx %d)", qdbidx, qdbidx);
  cmgb_ctx *c = m->ctx;
  DevTrPlan &dp = m->trplans[qdbidx][alg];
  const int wantT = c->tile_rows ? c->tile_rows : 16;
  const int wantA = c->arena;
  if (dp.built && dp.T == wantT && dp.nt == c->threads && dp.arena == wantA) { *ret = &dp; return CMGB_OK; }
  if (dp.d_states) { cudaFree(dp.d_states); dp.d_states = nullptr; }
  TrPlanOut po;
  int T = wantT;
  for (;;) {
    po = TrPlanOut();
    // arena: 1 shared memory, 2 global memory, 0 shared when it fits the device, else global
    bool gl = wantA == 2;
    if (!build_tr_plan(&m->desc, qdbidx, T, c->threads, alg == 1, gl, &po)) ERRF(CMGB_EINCOMPAT, "%s", po.err.c_str());
    if (!gl && wantA == 0 && po.plan.smem_bytes + 64 > c->max_smem_optin) {
      po = TrPlanOut();
      if (!build_tr_plan(&m->desc, qdbidx, T, c->threads, alg == 1, true, &po)) ERRF(CMGB_EINCOMPAT, "%s", po.err.c_str());
    }
    if (po.plan.smem_bytes + 64 <= c->max_smem_optin) break;
    if (T <= 2) ERRF(CMGB_ERANGE, "model needs %d bytes of shared memory per CTA even with 2-row tiles", po.plan.smem_bytes);
    T = T > 8 ? T - 4 : T - 2;
  }
  CUDA_TRY(cudaMalloc(&dp.d_states, sizeof(TrStateInfo) * po.phases.size()));
  CUDA_TRY(cudaMemcpy(dp.d_states, po.phases.data(), sizeof(TrStateInfo) * po.phases.size(), cudaMemcpyHostToDevice));
  dp.plan = po.plan;
  dp.T = wantT;
  dp.nt = c->threads;
  dp.arena = wantA;
  dp.built = true;
  *ret = &dp;
  return CMGB_OK;
}

// Common driver of the truncated scanners.  alg: 0 TrCYK (float), 1 integer
// TrInside.  The kernel reports, per window, the root cells that set a new
// running maximum within the window; cells are kept when they also beat the
// maxima of every earlier window (the reference's sequential root test,
// src/cm_dpsearch_trunc.c:548-605), then resolved per end position.
static int scan_tr(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int pass_idx, int alg,
                   const uint8_t *host_dsq, const uint8_t *dev_dsq_in, int64_t i0, int64_t j0,
                   float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                   int64_t *ret_envi, int64_t *ret_envj, float *ret_vsc, int *ret_mode, float *ret_sc)
{
  const char *fn = alg == 1 ? "RefITrInsideScan" : "RefTrCYKScan";
  if (!c || !m) ERRF(CMGB_EINVAL, "%s, NULL context or model", fn);
  int fill_L = 0, fill_R = 0, fill_T = 0, pty_idx = -1;   // cm_TrFillFromPassIdx / cm_tr_penalties_IdxForPass
  switch (pass_idx) {
  case CMGB_PASS_5P_AND_3P_FORCE: case CMGB_PASS_5P_AND_3P_ANY: fill_L = fill_R = fill_T = 1; pty_idx = 0; break;
  case CMGB_PASS_5P_ONLY_FORCE: fill_R = 1; pty_idx = 1; break;
  case CMGB_PASS_3P_ONLY_FORCE: fill_L = 1; pty_idx = 2; break;
  default: ERRF(CMGB_EINVAL, "%s(), unexpected pass idx: %d", fn, pass_idx);
  }
  if (j0 < i0) ERRF(CMGB_EINCOMPAT, "%s, i0: %lld j0: %lld", fn, (long long) i0, (long long) j0);
  if (i0 < 1) ERRF(CMGB_EINCOMPAT, "%s, i0 must be >= 1", fn);
  if (host_dsq == nullptr && dev_dsq_in == nullptr) ERRF(CMGB_EINCOMPAT, "%s, dsq is NULL", fn);
  if (qdbidx < 0 || qdbidx > 2) ERRF(CMGB_EINCOMPAT, "%s, qdbidx is invalid", fn);
  if (!m->has_tr) ERRF(CMGB_EINCOMPAT, "%s, the model was created without truncation tables", fn);
  int st;
  CUDA_TRY(cudaSetDevice(c->device));
  DevTrPlan *dp;
  if ((st = get_tr_plan(m, qdbidx, alg, &dp, errbuf)) != CMGB_OK) return st;
  const ScanPlan &P = dp->plan;
  const int64_t L = j0 - i0 + 1;
  const int W = m->W;

  const unsigned char *d_dsq;
  int64_t lo = i0 - W - 1; if (lo < 0) lo = 0;
  if (dev_dsq_in) d_dsq = dev_dsq_in;
  else {
    size_t need = (size_t) (j0 + 2 - lo);
    if ((st = grow((void **) &c->d_dsq, &c->dsq_bytes, need, errbuf)) != CMGB_OK) return st;
    CUDA_TRY(cudaMemcpyAsync(c->d_dsq, host_dsq + lo, need, cudaMemcpyHostToDevice, c->stream));
    d_dsq = c->d_dsq - lo;
  }
  c->last_h2d = (dev_dsq_in ? 0 : (int64_t) (j0 + 2 - lo)) + (int64_t) sizeof(Control);

  const bool gl = P.arena_global != 0;
  // the kernel's dynamic shared-memory limit is set for every plan (an
  // explicit CTA count skips only the occupancy query's answer)
  int cps = c->ctas_per_sm;
#ifndef CMGB_HOST_EMULATION
  {
    int nb = 1;
    CUDA_TRY(prepare_tr_any(alg, gl, c->threads, P.smem_bytes, &nb));
    if (cps == 0) cps = nb < 1 ? 1 : nb;
  }
#else
  if (cps == 0) cps = 1;
#endif
  const int grid_max = c->nsm * cps;
  int64_t win = c->window_len;
  if (win <= 0) {
    win = (L + grid_max - 1) / grid_max;
    if (win < 8LL * W) win = 8LL * W;
  }
  // a window's root cells are numbered (row, length, mode) in 32 bits
  const int64_t win_cap = ((int64_t) 1 << 30) / (W + 1);
  if (win > win_cap) win = win_cap;
  win = ((win + P.T - 1) / P.T) * P.T;
  if (win > win_cap) win -= P.T;
  const int64_t nwin = (L + win - 1) / win;
  if (nwin > (1 << 24)) ERRF(CMGB_ERANGE, "%s, too many windows", fn);
  const int grid = (int) std::min<int64_t>(nwin, grid_max);

  const int accw = P.acc_w;
  size_t carry_need = sizeof(float) * 2 * (size_t) P.carry_elems * grid;
  size_t ring_need = sizeof(float) * (size_t) P.ring_elems * grid;
  if ((st = grow((void **) &c->d_carry, &c->carry_bytes, carry_need, errbuf)) != CMGB_OK) return st;
  if ((st = grow((void **) &c->d_ring, &c->ring_bytes, ring_need, errbuf)) != CMGB_OK) return st;
  if (gl && (st = grow((void **) &c->d_arena, &c->arena_bytes, sizeof(float) * (size_t) P.arena_elems * grid, errbuf)) != CMGB_OK) return st;
  int cand_cap = 0;
  if ((st = tr_cand_reserve(c, kTrCandCap, &cand_cap, errbuf)) != CMGB_OK) return st;
  if ((st = grow((void **) &c->d_winbest, &c->winbest_bytes, sizeof(unsigned long long) * (size_t) nwin, errbuf)) != CMGB_OK) return st;
  if ((st = grow((void **) &c->d_wmax, &c->wmax_bytes, sizeof(float) * 8 * (size_t) accw * nwin, errbuf)) != CMGB_OK) return st;
  if (ret_vsc && c->vsc_len < m->M) {
    cudaFree(c->d_vsc); c->d_vsc = nullptr;
    if (cudaMalloc(&c->d_vsc, sizeof(unsigned) * m->M) != cudaSuccess) ERRF(CMGB_EMEM, "out of device memory");
    c->vsc_len = m->M;
  }
  const bool greedy = !(m->flags & CMGB_NOTGREEDY);
  Control *h = c->h_ctl;
  std::vector<unsigned long long> winbest((size_t) nwin);
  std::vector<unsigned> vscu;
  for (int attempt = 0;; attempt++) {   // a second launch only when the candidate buffer was too small
  std::memset(h, 0, sizeof(Control));
  CUDA_TRY(cudaMemcpyAsync(c->d_ctl, h, sizeof(Control), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemsetAsync(c->d_winbest, 0, sizeof(unsigned long long) * (size_t) nwin, c->stream));
  if (ret_vsc) CUDA_TRY(cudaMemsetAsync(c->d_vsc, 0, sizeof(unsigned) * m->M, c->stream));

  TrKParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.st = dp->d_states; kp.plan = P; kp.arena = c->d_arena;
  kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc;
  kp.lmesc = m->d_lmesc; kp.rmesc = m->d_rmesc; kp.ilmesc = m->d_ilmesc; kp.irmesc = m->d_irmesc;
  kp.ilog = c->d_ilog;
  kp.dsq = d_dsq; kp.i0 = i0; kp.j0 = j0; kp.win_len = win; kp.nwin = (int) nwin;
  kp.queue = &c->d_ctl->queue; kp.carry = c->d_carry; kp.ring = c->d_ring;
  kp.cand = c->d_trcand; kp.ncand = &c->d_ctl->ncand; kp.cand_cap = cand_cap;
  kp.cand_cut = cutoff; kp.cand_pos = (hitlist && !greedy) ? 1 : 0;
  if (!hitlist) { kp.cand_cut = 3.0e38f; kp.cand_pos = 0; }
  kp.env_cut = (ret_envi || ret_envj) ? env_cutoff : 3.0e38f;
  kp.fill_L = fill_L; kp.fill_R = fill_R; kp.fill_T = fill_T; kp.pty_idx = pty_idx;
  kp.vsc = ret_vsc ? c->d_vsc : nullptr;
  kp.winbest = c->d_winbest; kp.wmax = c->d_wmax; kp.err = &c->d_ctl->err;

  const size_t smem = (size_t) P.smem_bytes;
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  launch_tr_any(alg, gl, grid, c->threads, smem, c->stream, kp);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  CUDA_TRY(cudaMemcpyAsync(h, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(winbest.data(), c->d_winbest, sizeof(unsigned long long) * (size_t) nwin, cudaMemcpyDeviceToHost, c->stream));
  if (ret_vsc) { vscu.resize(m->M); CUDA_TRY(cudaMemcpyAsync(vscu.data(), c->d_vsc, sizeof(unsigned) * m->M, cudaMemcpyDeviceToHost, c->stream)); }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  c->last_launches = attempt + 1;
  c->last_d2h = (int64_t) sizeof(Control) + (int64_t) sizeof(unsigned long long) * nwin + (ret_vsc ? (int64_t) sizeof(unsigned) * m->M : 0);
  if (!(h->err & 1)) break;
  if (attempt > 0) ERRF(CMGB_ERANGE, "%s, more than %d candidate root cells; raise the cutoff", fn, cand_cap);
  if ((st = tr_cand_reserve(c, (int64_t) h->ncand + h->ncand / 4, &cand_cap, errbuf)) != CMGB_OK) return st;
  }

  auto u2f = [](unsigned u) { if (u == 0) return CMGB_IMPOSSIBLE; unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u; float f; std::memcpy(&f, &b, 4); return f; };
  // best parse over all windows: highest score, earliest window on ties
  float best = CMGB_IMPOSSIBLE; int bmode = CMGB_TRMODE_UNKNOWN; bool any = false;
  for (int64_t w = 0; w < nwin; w++) {
    const unsigned long long k = winbest[(size_t) w];
    if (!k) continue;
    const float f = u2f((unsigned) (k >> 32));
    if (!any || f > best) {
      best = f; any = true;
      const unsigned pos = 0xFFFFFFFFu - (unsigned) (k & 0xFFFFFFFFULL);
      bmode = 3 - (int) (pos & 3u);
    }
  }
  if (ret_sc) *ret_sc = best;
  if (ret_mode) *ret_mode = bmode;
  if (ret_vsc) { for (int v = 0; v < m->M; v++) ret_vsc[v] = u2f(vscu[v]); ret_vsc[0] = best; }

  // candidates: keep the cells that beat the running maxima of all earlier windows
  const int n = h->ncand;
  std::vector<TrCand> tc((size_t) n);
  if (n > 0) CUDA_TRY(cudaMemcpy(tc.data(), c->d_trcand, sizeof(TrCand) * (size_t) n, cudaMemcpyDeviceToHost));
  c->last_d2h += (int64_t) sizeof(TrCand) * n;
  std::vector<int> wmx;
  if (n > 0 && nwin > 1) {
    wmx.resize((size_t) 8 * accw * nwin);
    CUDA_TRY(cudaMemcpy(wmx.data(), c->d_wmax, sizeof(int) * wmx.size(), cudaMemcpyDeviceToHost));
    c->last_d2h += (int64_t) sizeof(int) * (int64_t) wmx.size();
  }
  std::sort(tc.begin(), tc.end(), [](const TrCand &a, const TrCand &b) {
    if (a.win != b.win) return a.win < b.win;
    if (a.j != b.j) return a.j < b.j;
    if (a.d != b.d) return a.d < b.d;
    return a.mode > b.mode;   // J, L, R, T
  });
  const int imp_i = alg == 1 ? -CMGB_INFTY : 0;
  std::vector<int> prefix((size_t) 8 * accw);
  if (alg == 1) std::fill(prefix.begin(), prefix.end(), imp_i);
  else { float fi = CMGB_IMPOSSIBLE; int b; std::memcpy(&b, &fi, 4); std::fill(prefix.begin(), prefix.end(), b); }
  auto greater = [alg](int a, int b) {   // native comparison of two raw scores
    if (alg == 1) return a > b;
    float fa, fb; std::memcpy(&fa, &a, 4); std::memcpy(&fb, &b, 4); return fa > fb;
  };
  std::vector<CandHost> &out = c->h_cand;
  out.clear();
  int64_t envi = j0 + 1, envj = i0 - 1;
  size_t q = 0;
  int cur_w = 0;
  while (q < tc.size()) {
    while (cur_w < tc[q].win) {   // fold window cur_w's final maxima into the prefix
      for (int x = 0; x < 8 * accw; x++) {
        const int v = wmx[(size_t) cur_w * 8 * accw + x];
        if (greater(v, prefix[x])) prefix[x] = v;
      }
      cur_w++;
    }
    // one (j, d) cell: its globally registered modes, best score, then smallest state, then mode order
    size_t e = q;
    while (e < tc.size() && tc[e].win == tc[q].win && tc[e].j == tc[q].j && tc[e].d == tc[q].d) e++;
    int wq = -1;
    for (size_t x = q; x < e; x++) {
      const TrCand &t = tc[x];
      const int mi = 3 - t.mode, pq = (int) (t.j & 1);
      if (!greater(t.raw, prefix[(size_t) (mi * 2 + pq) * accw + t.d - 1])) continue;
      if (wq < 0 || t.f > tc[wq].f || (t.f == tc[wq].f && t.y < tc[wq].y)) wq = (int) x;
    }
    if (wq >= 0) {
      const TrCand &t = tc[wq];
      if (t.f >= env_cutoff) { envi = std::min<int64_t>(envi, t.j - t.d + 1); envj = std::max<int64_t>(envj, t.j); }
      if (hitlist) { CandHost ch; ch.j = t.j; ch.d = t.d; ch.sc = t.f; ch.r = t.y; ch.mode = t.mode; out.push_back(ch); }
    }
    q = e;
  }
  if (ret_envi) *ret_envi = (envi == j0 + 1) ? -1 : envi;
  if (ret_envj) *ret_envj = (envj == i0 - 1) ? -1 : envj;

  if (hitlist) {
    std::vector<uint8_t> res_copy;
    const uint8_t *hd = host_dsq;
    if (do_null3 && !out.empty() && hd == nullptr) {
      res_copy.resize((size_t) (j0 + 2));
      CUDA_TRY(cudaMemcpy(res_copy.data() + i0, dev_dsq_in + i0, (size_t) L, cudaMemcpyDeviceToHost));
      c->last_d2h += L;
      hd = res_copy.data();
    }
    TruncFilter tf;
    tf.pass_idx = pass_idx; tf.local = (m->flags & CMGB_LOCAL_BEGIN) ? 1 : 0; tf.clen = m->clen;
    tf.ndidx = m->ndidx.data(); tf.ndtype = m->ndtype.data(); tf.lpos = m->emap_lpos.data(); tf.rpos = m->emap_rpos.data();
    ResolveArgs ra;
    ra.null = m->null.data(); ra.K = m->K; ra.null3_omega = m->null3_omega; ra.do_null3 = do_null3;
    ra.greedy = greedy ? 1 : 0; ra.cutoff = cutoff; ra.i0 = i0; ra.j0 = j0; ra.dsq = hd; ra.tr = &tf;
    resolve_hits(out, ra, hitlist->h);
  }
  return CMGB_OK;
}

extern "C" int cmgb_RefTrCYKScan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int pass_idx, const uint8_t *dsq,
                                 int64_t i0, int64_t j0, float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff,
                                 int64_t *envi, int64_t *envj, float *vsc, int *mode, float *sc)
{
  if (dsq == nullptr) ERRF(CMGB_EINCOMPAT, "RefTrCYKScan, dsq is NULL");
  return scan_tr(c, m, errbuf, qdbidx, pass_idx, 0, dsq, nullptr, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, mode, sc);
}
extern "C" int cmgb_RefITrInsideScan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int pass_idx, const uint8_t *dsq,
                                     int64_t i0, int64_t j0, float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff,
                                     int64_t *envi, int64_t *envj, float *vsc, int *mode, float *sc)
{
  if (dsq == nullptr) ERRF(CMGB_EINCOMPAT, "RefITrInsideScan, dsq is NULL");
  return scan_tr(c, m, errbuf, qdbidx, pass_idx, 1, dsq, nullptr, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, mode, sc);
}
extern "C" int cmgb_RefTrCYKScan_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int pass_idx, const uint8_t *d_dsq,
                                     int64_t i0, int64_t j0, float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff,
                                     int64_t *envi, int64_t *envj, float *vsc, int *mode, float *sc)
{
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "RefTrCYKScan, dsq is NULL");
  return scan_tr(c, m, errbuf, qdbidx, pass_idx, 0, nullptr, d_dsq, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, mode, sc);
}
extern "C" int cmgb_RefITrInsideScan_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx, int pass_idx, const uint8_t *d_dsq,
                                         int64_t i0, int64_t j0, float cutoff, cmgb_hitlist *hl, int do_null3, float env_cutoff,
                                         int64_t *envi, int64_t *envj, float *vsc, int *mode, float *sc)
{
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "RefITrInsideScan, dsq is NULL");
  return scan_tr(c, m, errbuf, qdbidx, pass_idx, 1, nullptr, d_dsq, i0, j0, cutoff, hl, do_null3, env_cutoff, envi, envj, vsc, mode, sc);
}

// ---------------------------------------------------------------------------
// Batched scans: n independent sequences of one model in one persistent
// launch, one work item per sequence, longest first.
// seqs: host residues (copied to the device per call) or, when d_seqs is
// given, residues already in device memory (host copies of single sequences
// are fetched only for the NULL3 composition of sequences with candidates).
// Owned rows per window of a batched scan: up to max(8 W, 2048), and no more
// than the batch's rows per resident CTA (at least W), so that a batch of few
// long sequences still spreads over every SM: a later window starts W-1 rows
// early, which leaves every cell's value unchanged.
static int64_t batch_window_len(const cmgb_ctx *c, int W, int64_t rows)
{
  const int64_t cap = std::max<int64_t>(8LL * W, 2048);
  const int64_t ctas = (int64_t) c->nsm * std::max(1, c->ctas_per_sm);
  const int64_t share = std::max<int64_t>(W, (rows + ctas - 1) / std::max<int64_t>(1, ctas));
  return std::min(cap, share);
}

static int scan_batch(cmgb_ctx *c, cmgb_model *m, char *errbuf, int algo, int qdbidx, int pass_idx,
                      const uint8_t *seqs, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                      const int64_t *lengths, int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                      int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode);

extern "C" int cmgb_ScanBatch(cmgb_ctx *c, cmgb_model *m, char *errbuf, int algo, int qdbidx, int pass_idx,
                              const uint8_t *seqs, int64_t seqs_len, const int64_t *offsets, const int64_t *lengths,
                              int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                              int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode)
{
  if (seqs == nullptr) ERRF(CMGB_EINCOMPAT, "ScanBatch, no sequences");
  return scan_batch(c, m, errbuf, algo, qdbidx, pass_idx, seqs, nullptr, seqs_len, offsets, lengths, nseq, cutoff, hitlist,
                    do_null3, env_cutoff, ret_nhits, ret_envi, ret_envj, ret_sc, ret_mode);
}

extern "C" int cmgb_ScanBatch_dev(cmgb_ctx *c, cmgb_model *m, char *errbuf, int algo, int qdbidx, int pass_idx,
                                  const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets, const int64_t *lengths,
                                  int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                                  int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode)
{
  if (d_seqs == nullptr) ERRF(CMGB_EINCOMPAT, "ScanBatch, no sequences");
  return scan_batch(c, m, errbuf, algo, qdbidx, pass_idx, nullptr, d_seqs, seqs_len, offsets, lengths, nseq, cutoff, hitlist,
                    do_null3, env_cutoff, ret_nhits, ret_envi, ret_envj, ret_sc, ret_mode);
}

static int scan_batch(cmgb_ctx *c, cmgb_model *m, char *errbuf, int algo, int qdbidx, int pass_idx,
                      const uint8_t *seqs, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                      const int64_t *lengths, int nseq, float cutoff, cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                      int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc, int *ret_mode)
{
  static const char *fn = "ScanBatch";
  if (!c || !m) ERRF(CMGB_EINVAL, "%s, NULL context or model", fn);
  if (algo < CMGB_ALGO_CYK || algo > CMGB_ALGO_ITRINSIDE) ERRF(CMGB_EINVAL, "%s, unknown algorithm %d", fn, algo);
  if ((seqs == nullptr && d_seqs == nullptr) || offsets == nullptr || lengths == nullptr || nseq < 1)
    ERRF(CMGB_EINCOMPAT, "%s, no sequences", fn);
  if (qdbidx < 0 || qdbidx > 2) ERRF(CMGB_EINCOMPAT, "%s, qdbidx is invalid", fn);
  const bool tr = algo >= CMGB_ALGO_TRCYK;
  const int alg = tr ? algo - CMGB_ALGO_TRCYK : algo;
  int fill_L = 0, fill_R = 0, fill_T = 0, pty_idx = 0;
  if (tr) {
    switch (pass_idx) {
    case CMGB_PASS_5P_AND_3P_FORCE: case CMGB_PASS_5P_AND_3P_ANY: fill_L = fill_R = fill_T = 1; pty_idx = 0; break;
    case CMGB_PASS_5P_ONLY_FORCE: fill_R = 1; pty_idx = 1; break;
    case CMGB_PASS_3P_ONLY_FORCE: fill_L = 1; pty_idx = 2; break;
    default: ERRF(CMGB_EINVAL, "%s, unexpected pass idx: %d", fn, pass_idx);
    }
    if (!m->has_tr) ERRF(CMGB_EINCOMPAT, "%s, the model was created without truncation tables", fn);
  }
  for (int q = 0; q < nseq; q++)   // sentinel, lengths[q] residues, sentinel, all inside the buffer
    if (!(lengths[q] >= 1 && offsets[q] >= 0 && offsets[q] + lengths[q] + 1 <= seqs_len - 1))
      ERRF(CMGB_EINCOMPAT, "%s, sequence %d lies outside the buffer", fn, q);
  int st;
  CUDA_TRY(cudaSetDevice(c->device));
  const ScanPlan *P;
  const void *d_states = nullptr;
  const unsigned char *d_rec = nullptr;
  if (tr) { DevTrPlan *dp; if ((st = get_tr_plan(m, qdbidx, alg, &dp, errbuf)) != CMGB_OK) return st; P = &dp->plan; d_states = dp->d_states; }
  else { DevPlan *dp; if ((st = get_plan(m, qdbidx, alg, &dp, errbuf)) != CMGB_OK) return st; P = &dp->plan; d_states = dp->d_states; d_rec = dp->d_rec; }

  // work items: one per sequence for the truncated scanners; the standard
  // scanners cut sequences longer than a window into windows that start W-1
  // rows early (as the single-sequence scan does).  Longest first.
  const int64_t wlen = batch_window_len(c, m->W, std::accumulate(lengths, lengths + nseq, (int64_t) 0));
  std::vector<int> wseq;                 // sequence of each window
  std::vector<long long> ws, we, ws0;
  for (int q = 0; q < nseq; q++) {
    const int64_t a = offsets[q] + 1, b = offsets[q] + lengths[q];
    if (tr || lengths[q] <= wlen) { wseq.push_back(q); ws.push_back(a); we.push_back(b); ws0.push_back(a); continue; }
    for (int64_t s = a; s <= b; s += wlen) {
      wseq.push_back(q); ws.push_back(s); we.push_back(std::min<int64_t>(b, s + wlen - 1));
      ws0.push_back(std::max<int64_t>(a, s - (m->W - 1)));
    }
  }
  if (wseq.size() > (size_t) (1 << 24)) ERRF(CMGB_ERANGE, "%s, too many windows", fn);
  const int nw = (int) wseq.size();
  std::vector<int> order(nw);
  for (int w = 0; w < nw; w++) order[w] = w;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return we[a] - ws0[a] > we[b] - ws0[b]; });
  {
    std::vector<long long> a(nw), b(nw), c(nw); std::vector<int> sq(nw);
    for (int w = 0; w < nw; w++) { a[w] = ws[order[w]]; b[w] = we[order[w]]; c[w] = ws0[order[w]]; sq[w] = wseq[order[w]]; }
    ws.swap(a); we.swap(b); ws0.swap(c); wseq.swap(sq);
  }
  // one device block: residues, window ranges, per-window outputs
  auto al = [](size_t x) { return (x + 255) & ~(size_t) 255; };
  const size_t o_ws = d_seqs ? 0 : al((size_t) seqs_len), o_we = o_ws + al(sizeof(long long) * nw), o_ws0 = o_we + al(sizeof(long long) * nw);
  const size_t o_out = o_ws0 + al(sizeof(long long) * nw);
  const size_t out_bytes = tr ? sizeof(unsigned long long) * nw : sizeof(long long) * 2 * nw + sizeof(unsigned) * nw;
  if ((st = grow((void **) &c->d_dsq, &c->dsq_bytes, o_out + al(out_bytes), errbuf)) != CMGB_OK) return st;
  unsigned char *blk = c->d_dsq;
  std::vector<unsigned char> out_init(out_bytes, 0);
  if (!tr) {
    long long *env = reinterpret_cast<long long *>(out_init.data());
    for (int w = 0; w < nw; w++) { env[2 * w] = LLONG_MAX; env[2 * w + 1] = -1; }
  }
  if (!d_seqs) CUDA_TRY(cudaMemcpyAsync(blk, seqs, (size_t) seqs_len, cudaMemcpyHostToDevice, c->stream));
  const unsigned char *res = d_seqs ? d_seqs : blk;
  CUDA_TRY(cudaMemcpyAsync(blk + o_ws, ws.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(blk + o_we, we.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(blk + o_ws0, ws0.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(blk + o_out, out_init.data(), out_bytes, cudaMemcpyHostToDevice, c->stream));
  c->last_h2d = (d_seqs ? 0 : seqs_len) + (int64_t) (3 * sizeof(long long) * nw + out_bytes + sizeof(Control));

  const bool gl = P->arena_global != 0;
  // the kernel's dynamic shared-memory limit is set for every plan (an
  // explicit CTA count skips only the occupancy query's answer)
  int cps = c->ctas_per_sm;
#ifndef CMGB_HOST_EMULATION
  {
    int nb = 1;
    if (tr) CUDA_TRY(prepare_tr_any(alg, gl, c->threads, P->smem_bytes, &nb));
    else CUDA_TRY(prepare_any(alg, gl, c->threads, P->smem_bytes, &nb));
    if (cps == 0) cps = nb < 1 ? 1 : nb;
  }
#else
  if (cps == 0) cps = 1;
#endif
  const int grid = std::min(nw, c->nsm * cps);
  if ((st = grow((void **) &c->d_carry, &c->carry_bytes, sizeof(float) * 2 * (size_t) P->carry_elems * grid, errbuf)) != CMGB_OK) return st;
  if ((st = grow((void **) &c->d_ring, &c->ring_bytes, sizeof(float) * (size_t) P->ring_elems * grid, errbuf)) != CMGB_OK) return st;
  if (gl && (st = grow((void **) &c->d_arena, &c->arena_bytes, sizeof(float) * (size_t) P->arena_elems * grid, errbuf)) != CMGB_OK) return st;
  int cand_cap = c->cand_cap;
  if (tr && (st = tr_cand_reserve(c, kTrCandCap, &cand_cap, errbuf)) != CMGB_OK) return st;
  Control *h = c->h_ctl;
  std::vector<unsigned char> outv(out_bytes);
  const bool greedy = !(m->flags & CMGB_NOTGREEDY);
  const float ccut = hitlist ? cutoff : 3.0e38f;
  const int cpos = (hitlist && !greedy) ? 1 : 0;
  const float ecut = (ret_envi || ret_envj) ? env_cutoff : 3.0e38f;
  for (int attempt = 0;; attempt++) {   // a second launch only when the candidate buffer was too small
  std::memset(h, 0, sizeof(Control));
  CUDA_TRY(cudaMemcpyAsync(c->d_ctl, h, sizeof(Control), cudaMemcpyHostToDevice, c->stream));
  if (attempt > 0) CUDA_TRY(cudaMemcpyAsync(blk + o_out, out_init.data(), out_bytes, cudaMemcpyHostToDevice, c->stream));

  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  if (tr) {
    TrKParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.st = (const TrStateInfo *) d_states; kp.plan = *P; kp.arena = c->d_arena;
    kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc;
    kp.lmesc = m->d_lmesc; kp.rmesc = m->d_rmesc; kp.ilmesc = m->d_ilmesc; kp.irmesc = m->d_irmesc;
    kp.ilog = c->d_ilog;
    kp.dsq = res; kp.i0 = 1; kp.j0 = seqs_len - 2; kp.win_len = 0; kp.nwin = nw;
    kp.queue = &c->d_ctl->queue; kp.carry = c->d_carry; kp.ring = c->d_ring;
    kp.cand = c->d_trcand; kp.ncand = &c->d_ctl->ncand; kp.cand_cap = cand_cap;
    kp.cand_cut = ccut; kp.cand_pos = cpos; kp.env_cut = ecut;
    kp.fill_L = fill_L; kp.fill_R = fill_R; kp.fill_T = fill_T; kp.pty_idx = pty_idx;
    kp.vsc = nullptr; kp.winbest = reinterpret_cast<unsigned long long *>(blk + o_out); kp.wmax = nullptr;
    kp.err = &c->d_ctl->err;
    kp.win_s = reinterpret_cast<const long long *>(blk + o_ws); kp.win_e = reinterpret_cast<const long long *>(blk + o_we);
    launch_tr_any(alg, gl, grid, c->threads, (size_t) P->smem_bytes, c->stream, kp);
  } else {
    KParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.st = (const StateInfo *) d_states; kp.plan = *P; kp.rec = d_rec; kp.arena = c->d_arena;
    kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc; kp.ilog = c->d_ilog; kp.flog = c->d_flog;
    kp.dsq = res; kp.i0 = 1; kp.j0 = seqs_len - 2; kp.win_len = 0; kp.nwin = nw;
    kp.queue = &c->d_ctl->queue; kp.carry = c->d_carry; kp.ring = c->d_ring;
    kp.cand = c->d_cand; kp.ncand = &c->d_ctl->ncand; kp.cand_cap = cand_cap;
    kp.cand_cut = ccut; kp.cand_pos = cpos; kp.env_cut = ecut;
    kp.env = reinterpret_cast<long long *>(blk + o_out);
    kp.best = reinterpret_cast<unsigned *>(blk + o_out + sizeof(long long) * 2 * nw);
    kp.vsc = nullptr; kp.err = &c->d_ctl->err;
    kp.win_s = reinterpret_cast<const long long *>(blk + o_ws); kp.win_e = reinterpret_cast<const long long *>(blk + o_we);
    kp.win_s0 = reinterpret_cast<const long long *>(blk + o_ws0);
    launch_any(alg, gl, grid, c->threads, (size_t) P->smem_bytes, c->stream, kp);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  CUDA_TRY(cudaMemcpyAsync(h, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(outv.data(), blk + o_out, out_bytes, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  c->last_launches = attempt + 1;
  c->last_d2h = (int64_t) (sizeof(Control) + out_bytes);
  if (h->err & 2) ERRF(CMGB_ENODEV, "%s, a bounded device wait ran out (phase record copy)", fn);
  if (!(h->err & 1)) break;
  if (attempt > 0) ERRF(CMGB_ERANGE, "%s, more than %d candidate root cells; raise the cutoff", fn, cand_cap);
  const int64_t need = (int64_t) h->ncand + h->ncand / 4;
  if (tr) { if ((st = tr_cand_reserve(c, need, &cand_cap, errbuf)) != CMGB_OK) return st; }
  else {   // grow the standard candidate buffer (kept for later calls)
    if (need > kTrCandMax) ERRF(CMGB_ERANGE, "%s, more than %lld candidate root cells; raise the cutoff", fn, (long long) kTrCandMax);
    cudaFree(c->d_cand); c->d_cand = nullptr; c->cand_cap = 0;
    if (cudaMalloc(&c->d_cand, sizeof(Cand) * (size_t) need) != cudaSuccess) ERRF(CMGB_EMEM, "%s, out of device memory for candidates", fn);
    c->cand_cap = cand_cap = (int) need;
  }
  }
  auto u2f = [](unsigned u) { if (u == 0) return CMGB_IMPOSSIBLE; unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u; float f; std::memcpy(&f, &b, 4); return f; };

  // per-sequence candidate lists (absolute coordinates in the buffer)
  const int n = h->ncand;
  std::vector<std::vector<CandHost>> per(nseq);
  std::vector<int64_t> envi(nseq), envj(nseq);
  for (int q = 0; q < nseq; q++) { envi[q] = offsets[q] + lengths[q] + 1; envj[q] = offsets[q]; }
  if (tr) {
    std::vector<TrCand> tc((size_t) n);
    if (n > 0) CUDA_TRY(cudaMemcpy(tc.data(), c->d_trcand, sizeof(TrCand) * (size_t) n, cudaMemcpyDeviceToHost));
    c->last_d2h += (int64_t) sizeof(TrCand) * n;
    std::sort(tc.begin(), tc.end(), [](const TrCand &a, const TrCand &b) {
      if (a.j != b.j) return a.j < b.j;
      if (a.d != b.d) return a.d < b.d;
      return a.mode > b.mode;
    });
    size_t q = 0;
    while (q < tc.size()) {   // each cell registered within its own (whole-sequence) window: keep the best mode
      size_t e = q, wq = q;
      while (e < tc.size() && tc[e].j == tc[q].j && tc[e].d == tc[q].d) {
        if (tc[e].f > tc[wq].f || (tc[e].f == tc[wq].f && tc[e].y < tc[wq].y)) wq = e;
        e++;
      }
      const TrCand &t = tc[wq];
      const int sq = wseq[t.win];
      if (t.f >= env_cutoff) { envi[sq] = std::min<int64_t>(envi[sq], t.j - t.d + 1); envj[sq] = std::max<int64_t>(envj[sq], t.j); }
      if (hitlist) { CandHost ch; ch.j = t.j; ch.d = t.d; ch.sc = t.f; ch.r = t.y; ch.mode = t.mode; per[sq].push_back(ch); }
      q = e;
    }
    const unsigned long long *wb = reinterpret_cast<const unsigned long long *>(outv.data());
    for (int w = 0; w < nw; w++) {
      const int sq = wseq[w];
      const unsigned long long k = wb[w];
      if (ret_sc) ret_sc[sq] = k ? u2f((unsigned) (k >> 32)) : CMGB_IMPOSSIBLE;
      if (ret_mode) ret_mode[sq] = k ? 3 - (int) ((0xFFFFFFFFu - (unsigned) (k & 0xFFFFFFFFULL)) & 3u) : CMGB_TRMODE_UNKNOWN;
    }
  } else {
    if (hitlist && n > 0) {
      c->h_cand.resize((size_t) n);
      CUDA_TRY(cudaMemcpy(c->h_cand.data(), c->d_cand, sizeof(Cand) * (size_t) n, cudaMemcpyDeviceToHost));
      c->last_d2h += (int64_t) sizeof(Cand) * n;
      std::vector<int> by_off(nseq);
      for (int q = 0; q < nseq; q++) by_off[q] = q;
      std::sort(by_off.begin(), by_off.end(), [&](int a, int b) { return offsets[a] < offsets[b]; });
      std::vector<long long> soff(nseq);
      for (int q = 0; q < nseq; q++) soff[q] = offsets[by_off[q]];
      // each candidate to its sequence (the last whose offset is below j);
      // contiguous slices of the candidates on host threads, each into its own
      // per-sequence lists, appended in slice order (the serial order)
      const size_t ncand = c->h_cand.size();
      const int nsl = nseq <= 4096 ? (int) std::min<size_t>(16, std::max<size_t>(1, ncand / 65536)) : 1;
      std::vector<std::vector<std::vector<CandHost>>> part((size_t) nsl, std::vector<std::vector<CandHost>>((size_t) nseq));
      parallel_for(nsl, [&](int t) {
        const size_t a = ncand * (size_t) t / (size_t) nsl, b = ncand * (size_t) (t + 1) / (size_t) nsl;
        for (size_t k = a; k < b; k++) {
          const CandHost &ch = c->h_cand[k];
          int lo = 0, hi = nseq - 1;
          while (lo < hi) { const int mid = (lo + hi + 1) / 2; if (soff[mid] < ch.j) lo = mid; else hi = mid - 1; }
          CandHost x = ch; x.mode = CMGB_TRMODE_J;
          part[t][by_off[lo]].push_back(x);
        }
      });
      for (int q = 0; q < nseq; q++)
        for (int t = 0; t < nsl; t++) per[q].insert(per[q].end(), part[t][q].begin(), part[t][q].end());
    }
    const long long *env = reinterpret_cast<const long long *>(outv.data());
    const unsigned *best = reinterpret_cast<const unsigned *>(outv.data() + sizeof(long long) * 2 * nw);
    std::vector<unsigned> bestq(nseq, 0u);
    for (int w = 0; w < nw; w++) {   // a long sequence's windows: union of envelopes, best of scores
      const int sq = wseq[w];
      if (env[2 * w + 1] >= 0) { envi[sq] = std::min<int64_t>(envi[sq], env[2 * w]); envj[sq] = std::max<int64_t>(envj[sq], env[2 * w + 1]); }
      bestq[sq] = std::max(bestq[sq], best[w]);
    }
    for (int q = 0; q < nseq; q++) {
      if (ret_sc) ret_sc[q] = u2f(bestq[q]);
      if (ret_mode) ret_mode[q] = CMGB_TRMODE_J;
    }
  }
  // device-resident residues: host copies of the sequences whose candidates need NULL3 compositions
  std::vector<uint8_t> hres;
  if (d_seqs && hitlist && do_null3) {
    for (int q = 0; q < nseq; q++) {
      if (per[q].empty()) continue;
      if (hres.empty()) hres.assign((size_t) seqs_len, (uint8_t) 255);
      CUDA_TRY(cudaMemcpy(hres.data() + offsets[q] + 1, d_seqs + offsets[q] + 1, (size_t) lengths[q], cudaMemcpyDeviceToHost));
      c->last_d2h += lengths[q];
    }
  }
  const uint8_t *hseq = d_seqs ? (hres.empty() ? nullptr : hres.data()) : seqs;
  // the sequences' hit lists are independent: resolve them on host threads,
  // then append them in sequence order
  std::vector<std::vector<cmgb_hit>> outq(hitlist ? nseq : 0);
  if (hitlist) {
    logsum_tables(nullptr, nullptr);
    TruncFilter tf;
    if (tr) {
      tf.pass_idx = pass_idx; tf.local = (m->flags & CMGB_LOCAL_BEGIN) ? 1 : 0; tf.clen = m->clen;
      tf.ndidx = m->ndidx.data(); tf.ndtype = m->ndtype.data(); tf.lpos = m->emap_lpos.data(); tf.rpos = m->emap_rpos.data();
    }
    parallel_for(nseq, [&](int q) {
      if (per[q].empty()) return;
      const int64_t off = offsets[q];
      ResolveArgs ra;
      ra.null = m->null.data(); ra.K = m->K; ra.null3_omega = m->null3_omega; ra.do_null3 = do_null3;
      ra.greedy = greedy ? 1 : 0; ra.cutoff = cutoff; ra.i0 = off + 1; ra.j0 = off + lengths[q]; ra.dsq = hseq;
      if (tr) ra.tr = &tf;
      resolve_hits(per[q], ra, outq[q]);
      for (cmgb_hit &h : outq[q]) { h.start -= off; h.stop -= off; }
    });
  }
  for (int q = 0; q < nseq; q++) {
    const int64_t off = offsets[q];
    if (ret_envi) ret_envi[q] = envj[q] < off + 1 ? -1 : envi[q] - off;
    if (ret_envj) ret_envj[q] = envj[q] < off + 1 ? -1 : envj[q] - off;
    if (hitlist) hitlist->h.insert(hitlist->h.end(), outq[q].begin(), outq[q].end());
    if (ret_nhits) ret_nhits[q] = hitlist ? (int64_t) outq[q].size() : 0;
  }
  return CMGB_OK;
}

// ---------------------------------------------------------------------------
// Multi-model batched scans: the windows of every (model, sequence) job in
// one work queue, one persistent launch per tile placement.
// seqs: host residues (copied per launch) or, when d_seqs is given,
// residues already in device memory (sequences whose candidates need NULL3
// compositions are read back individually).
static int scan_multi(cmgb_ctx *c, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                      int algo, int qdbidx, const uint8_t *seqs, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                      const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                      cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                      int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc);

extern "C" int cmgb_ScanMulti(cmgb_ctx *c, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                              int algo, int qdbidx, const uint8_t *seqs, int64_t seqs_len, const int64_t *offsets,
                              const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                              cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                              int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc)
{
  if (!seqs) ERRF(CMGB_EINCOMPAT, "ScanMulti, no jobs");
  return scan_multi(c, models, nmodels, cutoffs, errbuf, algo, qdbidx, seqs, nullptr, seqs_len, offsets, lengths, nseq,
                    job_model, job_seq, njobs, hitlist, do_null3, env_cutoff, ret_nhits, ret_envi, ret_envj, ret_sc);
}

extern "C" int cmgb_ScanMulti_dev(cmgb_ctx *c, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                                  int algo, int qdbidx, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                                  const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                                  cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                                  int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc)
{
  if (!d_seqs) ERRF(CMGB_EINCOMPAT, "ScanMulti, no jobs");
  return scan_multi(c, models, nmodels, cutoffs, errbuf, algo, qdbidx, nullptr, d_seqs, seqs_len, offsets, lengths, nseq,
                    job_model, job_seq, njobs, hitlist, do_null3, env_cutoff, ret_nhits, ret_envi, ret_envj, ret_sc);
}

static int scan_multi(cmgb_ctx *c, cmgb_model *const *models, int nmodels, const float *cutoffs, char *errbuf,
                      int algo, int qdbidx, const uint8_t *seqs, const uint8_t *d_seqs, int64_t seqs_len, const int64_t *offsets,
                      const int64_t *lengths, int nseq, const int *job_model, const int *job_seq, int njobs,
                      cmgb_hitlist *hitlist, int do_null3, float env_cutoff,
                      int64_t *ret_nhits, int64_t *ret_envi, int64_t *ret_envj, float *ret_sc)
{
  static const char *fn = "ScanMulti";
  if (!c || !models || nmodels < 1 || !cutoffs) ERRF(CMGB_EINVAL, "%s, NULL context, models or cutoffs", fn);
  if (algo < CMGB_ALGO_CYK || algo > CMGB_ALGO_FINSIDE) ERRF(CMGB_EINVAL, "%s, algorithm %d is not a standard scanner", fn, algo);
  if (qdbidx < 0 || qdbidx > 2) ERRF(CMGB_EINCOMPAT, "%s, qdbidx is invalid", fn);
  if ((!seqs && !d_seqs) || !offsets || !lengths || nseq < 1 || !job_model || !job_seq || njobs < 1) ERRF(CMGB_EINCOMPAT, "%s, no jobs", fn);
  for (int k = 0; k < nmodels; k++)
    if (!models[k] || models[k]->ctx != c) ERRF(CMGB_EINCOMPAT, "%s, model %d is NULL or belongs to another context", fn, k);
  for (int q = 0; q < nseq; q++)
    if (!(lengths[q] >= 1 && offsets[q] >= 0 && offsets[q] + lengths[q] + 1 <= seqs_len - 1))
      ERRF(CMGB_EINCOMPAT, "%s, sequence %d lies outside the buffer", fn, q);
  std::vector<int64_t> keys((size_t) njobs);
  for (int k = 0; k < njobs; k++) {
    if (job_model[k] < 0 || job_model[k] >= nmodels || job_seq[k] < 0 || job_seq[k] >= nseq)
      ERRF(CMGB_EINCOMPAT, "%s, job %d names model %d / sequence %d out of range", fn, k, job_model[k], job_seq[k]);
    keys[k] = (int64_t) job_model[k] * nseq + job_seq[k];
  }
  std::vector<int> by_key((size_t) njobs);
  for (int k = 0; k < njobs; k++) by_key[k] = k;
  std::sort(by_key.begin(), by_key.end(), [&](int a, int b) { return keys[a] < keys[b]; });
  for (int k = 1; k < njobs; k++)
    if (keys[by_key[k]] == keys[by_key[k - 1]]) ERRF(CMGB_EINCOMPAT, "%s, jobs %d and %d repeat a (model, sequence) pair", fn, by_key[k - 1], by_key[k]);
  auto job_of = [&](int mi, int q) {   // job index of (model, sequence)
    const int64_t key = (int64_t) mi * nseq + q;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) { const int mid = (lo + hi) / 2; if (keys[by_key[mid]] < key) lo = mid + 1; else hi = mid; }
    return keys[by_key[lo]] == key ? by_key[lo] : -1;
  };
  const int alg = algo;
  int st;
  CUDA_TRY(cudaSetDevice(c->device));
  std::vector<DevPlan *> plan((size_t) nmodels, nullptr);
  std::vector<double> rate((size_t) nmodels, 0.0);   // cells per residue of a full-length row
  std::vector<char> used((size_t) nmodels, 0);
  for (int k = 0; k < njobs; k++) used[job_model[k]] = 1;
  for (int mi = 0; mi < nmodels; mi++) {
    if (!used[mi]) continue;
    if ((st = get_plan(models[mi], qdbidx, alg, &plan[mi], errbuf)) != CMGB_OK) return st;
    const cmgb_model_desc *d = &models[mi]->desc;
    rate[mi] = (double) (cmgb_count_cells(d, qdbidx, d->W) - cmgb_count_cells(d, qdbidx, d->W - 1));
  }

  // windows of every job (as cmgb_ScanBatch cuts a sequence), with their cost
  struct Win { int job; long long s, e, s0; double cost; };
  std::vector<Win> all;
  int64_t job_rows = 0;
  for (int k = 0; k < njobs; k++) job_rows += lengths[job_seq[k]];
  for (int k = 0; k < njobs; k++) {
    const int mi = job_model[k], q = job_seq[k];
    const int Wm = models[mi]->W;
    const int64_t wlen = batch_window_len(c, Wm, job_rows);
    const int64_t a = offsets[q] + 1, b = offsets[q] + lengths[q];
    for (int64_t s0w = a; s0w <= b; s0w += wlen) {
      Win x; x.job = k; x.s = s0w; x.e = std::min<int64_t>(b, s0w + wlen - 1);
      x.s0 = s0w == a ? a : std::max<int64_t>(a, s0w - (Wm - 1));
      x.cost = rate[mi] * (double) (x.e - x.s0 + 1);
      all.push_back(x);
    }
  }
  if (all.size() > (size_t) (1 << 24)) ERRF(CMGB_ERANGE, "%s, too many windows", fn);

  std::vector<std::vector<CandHost>> per((size_t) njobs);
  std::vector<int64_t> envi((size_t) njobs), envj((size_t) njobs);
  std::vector<unsigned> bestj((size_t) njobs, 0u);
  for (int k = 0; k < njobs; k++) { const int q = job_seq[k]; envi[k] = offsets[q] + lengths[q] + 1; envj[k] = offsets[q]; }
  float total_ms = 0.f;
  int launches = 0;
  int64_t h2d = 0, d2h = 0;
  const float ecut = (ret_envi || ret_envj) ? env_cutoff : 3.0e38f;

  for (int glp = 0; glp < 2; glp++) {   // one launch per tile placement (shared, then global arena)
    std::vector<Win> wv;
    for (const Win &x : all) if ((plan[job_model[x.job]]->plan.arena_global != 0) == (glp == 1)) wv.push_back(x);
    if (wv.empty()) continue;
    std::stable_sort(wv.begin(), wv.end(), [](const Win &a, const Win &b) { return a.cost > b.cost; });
    const int nw = (int) wv.size();
    const bool gl = glp == 1;
    // the common per-CTA strides of this launch: largest over its models
    int max_elems = 0, max_carry = 0, max_ring = 0, max_arena = 0, smem = 0;
    std::vector<int> gmodels;
    for (int mi = 0; mi < nmodels; mi++) {
      if (!plan[mi] || (plan[mi]->plan.arena_global != 0) != gl) continue;
      bool has = false;
      for (const Win &x : wv) if (job_model[x.job] == mi) { has = true; break; }
      if (!has) continue;
      const ScanPlan &P = plan[mi]->plan;
      gmodels.push_back(mi);
      max_elems = std::max(max_elems, P.smem_elems); max_carry = std::max(max_carry, P.carry_elems);
      max_ring = std::max(max_ring, P.ring_elems); max_arena = std::max(max_arena, P.arena_elems);
    }
    smem = max_elems * 4 + 32;
    if (smem + 64 > c->max_smem_optin) ERRF(CMGB_ERANGE, "%s, %d bytes of shared memory per CTA exceed the device", fn, smem);

    auto al = [](size_t x) { return (x + 255) & ~(size_t) 255; };
    const size_t o_ws = d_seqs ? 0 : al((size_t) seqs_len), o_we = o_ws + al(sizeof(long long) * nw), o_ws0 = o_we + al(sizeof(long long) * nw);
    const size_t o_cm = o_ws0 + al(sizeof(long long) * nw), o_kp = o_cm + al(sizeof(int) * nw);
    const size_t o_out = o_kp + al(sizeof(KParams) * (size_t) nmodels);
    const size_t out_bytes = sizeof(long long) * 2 * nw + sizeof(unsigned) * nw;
    if ((st = grow((void **) &c->d_dsq, &c->dsq_bytes, o_out + al(out_bytes), errbuf)) != CMGB_OK) return st;
    unsigned char *blk = c->d_dsq;
    std::vector<long long> ws(nw), we(nw), ws0(nw);
    std::vector<int> icm(nw);
    for (int w = 0; w < nw; w++) { ws[w] = wv[w].s; we[w] = wv[w].e; ws0[w] = wv[w].s0; icm[w] = job_model[wv[w].job]; }
    std::vector<unsigned char> out_init(out_bytes, 0);
    {
      long long *env = reinterpret_cast<long long *>(out_init.data());
      for (int w = 0; w < nw; w++) { env[2 * w] = LLONG_MAX; env[2 * w + 1] = -1; }
    }
    // the kernel's dynamic shared-memory limit is set for every launch (an
    // explicit CTA count skips only the occupancy query's answer)
    int cps = c->ctas_per_sm;
#ifndef CMGB_HOST_EMULATION
    {
      int nb = 1;
      CUDA_TRY(prepare_any(alg, gl, c->threads, smem, &nb, true));
      if (cps == 0) cps = nb < 1 ? 1 : nb;
    }
#else
    if (cps == 0) cps = 1;
#endif
    const int grid = std::min(nw, c->nsm * cps);
    if ((st = grow((void **) &c->d_carry, &c->carry_bytes, sizeof(float) * 2 * (size_t) max_carry * grid, errbuf)) != CMGB_OK) return st;
    if ((st = grow((void **) &c->d_ring, &c->ring_bytes, sizeof(float) * (size_t) max_ring * grid, errbuf)) != CMGB_OK) return st;
    if (gl && (st = grow((void **) &c->d_arena, &c->arena_bytes, sizeof(float) * (size_t) max_arena * grid, errbuf)) != CMGB_OK) return st;
    if (c->cand_cap == 0) {
      if (cudaMalloc(&c->d_cand, sizeof(Cand) * (size_t) kCandCap) != cudaSuccess) ERRF(CMGB_EMEM, "%s, out of device memory for candidates", fn);
      c->cand_cap = kCandCap;
    }
    Control *h = c->h_ctl;
    std::vector<unsigned char> outv(out_bytes);
    std::vector<KParams> kps((size_t) nmodels);
    for (int attempt = 0;; attempt++) {   // a second launch only when the candidate buffer was too small
      std::memset(kps.data(), 0, sizeof(KParams) * kps.size());
      for (int mi : gmodels) {
        cmgb_model *m = models[mi];
        KParams &kp = kps[mi];
        const bool greedy = !(m->flags & CMGB_NOTGREEDY);
        kp.st = plan[mi]->d_states; kp.plan = plan[mi]->plan; kp.rec = plan[mi]->d_rec; kp.arena = c->d_arena;
        kp.plan.smem_elems = max_elems; kp.plan.carry_elems = max_carry; kp.plan.ring_elems = max_ring; kp.plan.arena_elems = max_arena;
        kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc; kp.ilog = c->d_ilog; kp.flog = c->d_flog;
        kp.dsq = d_seqs ? d_seqs : blk; kp.i0 = 1; kp.j0 = seqs_len - 2; kp.nwin = nw;
        kp.queue = &c->d_ctl->queue; kp.carry = c->d_carry; kp.ring = c->d_ring;
        kp.cand = c->d_cand; kp.ncand = &c->d_ctl->ncand; kp.cand_cap = c->cand_cap;
        kp.cand_cut = hitlist ? cutoffs[mi] : 3.0e38f; kp.cand_pos = (hitlist && !greedy) ? 1 : 0; kp.env_cut = ecut;
        kp.env = reinterpret_cast<long long *>(blk + o_out);
        kp.best = reinterpret_cast<unsigned *>(blk + o_out + sizeof(long long) * 2 * nw);
        kp.err = &c->d_ctl->err;
        kp.win_s = reinterpret_cast<const long long *>(blk + o_ws); kp.win_e = reinterpret_cast<const long long *>(blk + o_we);
        kp.win_s0 = reinterpret_cast<const long long *>(blk + o_ws0);
        kp.cand_tag = mi;
      }
      // launch parameters: the first model of the launch supplies the queue,
      // the window count and the common shared-memory layout
      KParams k0 = kps[gmodels[0]];
      k0.multi = reinterpret_cast<const KParams *>(blk + o_kp);
      k0.item_cm = reinterpret_cast<const int *>(blk + o_cm);
      std::memset(h, 0, sizeof(Control));
      if (!d_seqs) CUDA_TRY(cudaMemcpyAsync(blk, seqs, (size_t) seqs_len, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_ws, ws.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_we, we.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_ws0, ws0.data(), sizeof(long long) * nw, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_cm, icm.data(), sizeof(int) * nw, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_kp, kps.data(), sizeof(KParams) * kps.size(), cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(blk + o_out, out_init.data(), out_bytes, cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(c->d_ctl, h, sizeof(Control), cudaMemcpyHostToDevice, c->stream));
      h2d += (d_seqs ? 0 : seqs_len) + (int64_t) (3 * sizeof(long long) * nw + sizeof(int) * nw + sizeof(KParams) * kps.size() + out_bytes + sizeof(Control));
      CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
      launch_any(alg, gl, grid, c->threads, (size_t) smem, c->stream, k0, true);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
      CUDA_TRY(cudaMemcpyAsync(h, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(cudaMemcpyAsync(outv.data(), blk + o_out, out_bytes, cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(cudaStreamSynchronize(c->stream));
      float ms = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
      total_ms += ms;
      launches++;
      d2h += (int64_t) (sizeof(Control) + out_bytes);
      if (h->err & 2) ERRF(CMGB_ENODEV, "%s, a bounded device wait ran out (phase record copy)", fn);
      if (!(h->err & 1)) break;
      if (attempt > 0) ERRF(CMGB_ERANGE, "%s, more than %d candidate root cells; raise the cutoffs", fn, c->cand_cap);
      const int64_t need = (int64_t) h->ncand + h->ncand / 4;
      if (need > kTrCandMax) ERRF(CMGB_ERANGE, "%s, more than %lld candidate root cells; raise the cutoffs", fn, (long long) kTrCandMax);
      cudaFree(c->d_cand); c->d_cand = nullptr; c->cand_cap = 0;
      if (cudaMalloc(&c->d_cand, sizeof(Cand) * (size_t) need) != cudaSuccess) ERRF(CMGB_EMEM, "%s, out of device memory for candidates", fn);
      c->cand_cap = (int) need;
    }
    // candidates -> jobs: model from the tag, sequence from the position
    const int n = h->ncand;
    if (hitlist && n > 0) {
      d2h += (int64_t) sizeof(Cand) * n;
      std::vector<Cand> raw((size_t) n);
      CUDA_TRY(cudaMemcpy(raw.data(), c->d_cand, sizeof(Cand) * (size_t) n, cudaMemcpyDeviceToHost));
      // per model, its jobs' sequences by offset: sequences of different
      // models may overlap (each model scanning its own regions of one buffer)
      std::vector<std::vector<int>> mseq((size_t) nmodels);
      for (int k = 0; k < njobs; k++) mseq[job_model[k]].push_back(job_seq[k]);
      for (auto &v : mseq) std::sort(v.begin(), v.end(), [&](int a, int b) { return offsets[a] < offsets[b]; });
      for (int i = 0; i < n; i++) {
        const Cand &cc = raw[i];
        const std::vector<int> &sq = mseq[cc.pad];
        if (sq.empty()) ERRF(CMGB_EINCOMPAT, "%s, a candidate cell matches no job", fn);
        int lo = 0, hi = (int) sq.size() - 1;   // the model's last sequence whose offset is below j
        while (lo < hi) { const int mid = (lo + hi + 1) / 2; if (offsets[sq[mid]] < cc.j) lo = mid; else hi = mid - 1; }
        const int k = job_of(cc.pad, sq[lo]);
        if (k < 0) ERRF(CMGB_EINCOMPAT, "%s, a candidate cell matches no job", fn);
        CandHost x; x.j = cc.j; x.d = cc.d; x.sc = cc.sc; x.r = cc.r; x.mode = CMGB_TRMODE_J;
        per[k].push_back(x);
      }
    }
    const long long *env = reinterpret_cast<const long long *>(outv.data());
    const unsigned *best = reinterpret_cast<const unsigned *>(outv.data() + sizeof(long long) * 2 * nw);
    for (int w = 0; w < nw; w++) {
      const int k = wv[w].job;
      if (env[2 * w + 1] >= 0) { envi[k] = std::min<int64_t>(envi[k], env[2 * w]); envj[k] = std::max<int64_t>(envj[k], env[2 * w + 1]); }
      bestj[k] = std::max(bestj[k], best[w]);
    }
  }
  // device-resident residues: host copies of the sequences whose candidates need NULL3 compositions
  std::vector<uint8_t> hres;
  if (d_seqs && hitlist && do_null3) {
    std::vector<char> need((size_t) nseq, 0);
    for (int k = 0; k < njobs; k++) if (!per[k].empty()) need[job_seq[k]] = 1;
    for (int q = 0; q < nseq; q++) {
      if (!need[q]) continue;
      if (hres.empty()) hres.assign((size_t) seqs_len, (uint8_t) 255);
      CUDA_TRY(cudaMemcpy(hres.data() + offsets[q] + 1, d_seqs + offsets[q] + 1, (size_t) lengths[q], cudaMemcpyDeviceToHost));
      d2h += lengths[q];
    }
  }
  const uint8_t *hseq = d_seqs ? (hres.empty() ? nullptr : hres.data()) : seqs;
  c->last_ms = total_ms;
  c->last_launches = launches;
  c->last_h2d = h2d; c->last_d2h = d2h;
  auto u2f = [](unsigned u) { if (u == 0) return CMGB_IMPOSSIBLE; unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u; float f; std::memcpy(&f, &b, 4); return f; };
  // the jobs' hit lists are independent: resolve them on host threads, then
  // append them in job order
  std::vector<std::vector<cmgb_hit>> outk(hitlist ? njobs : 0);
  if (hitlist) {
    logsum_tables(nullptr, nullptr);
    parallel_for(njobs, [&](int k) {
      if (per[k].empty()) return;
      const int q = job_seq[k];
      cmgb_model *mk = models[job_model[k]];
      const int64_t off = offsets[q];
      ResolveArgs ra;
      ra.null = mk->null.data(); ra.K = mk->K; ra.null3_omega = mk->null3_omega; ra.do_null3 = do_null3;
      ra.greedy = (mk->flags & CMGB_NOTGREEDY) ? 0 : 1; ra.cutoff = cutoffs[job_model[k]];
      ra.i0 = off + 1; ra.j0 = off + lengths[q]; ra.dsq = hseq;
      resolve_hits(per[k], ra, outk[k]);
      for (cmgb_hit &h : outk[k]) { h.start -= off; h.stop -= off; }
    });
  }
  for (int k = 0; k < njobs; k++) {
    const int q = job_seq[k];
    const int64_t off = offsets[q];
    if (ret_sc) ret_sc[k] = u2f(bestj[k]);
    if (ret_envi) ret_envi[k] = envj[k] < off + 1 ? -1 : envi[k] - off;
    if (ret_envj) ret_envj[k] = envj[k] < off + 1 ? -1 : envj[k] - off;
    if (hitlist) hitlist->h.insert(hitlist->h.end(), outk[k].begin(), outk[k].end());
    if (ret_nhits) ret_nhits[k] = hitlist ? (int64_t) outk[k].size() : 0;
  }
  return CMGB_OK;
}

// Times candidate shapes (tile rows x arena placement) of band set qdbidx and
// algorithm (0 CYK, 1 integer Inside, 2 float Inside) on a seeded iid sample and keeps the
// fastest for this model; later scans that leave the shape to the library use it.
extern "C" int cmgb_autotune(cmgb_ctx *c, cmgb_model *m, int qdbidx, int algo, int64_t sample_len,
                             int *ret_tile_rows, int *ret_arena, char *errbuf)
{
  if (!c || !m || qdbidx < 0 || qdbidx > 2 || algo < 0 || algo > 2) ERRF(CMGB_EINVAL, "cmgb_autotune: invalid argument");
  // default sample: enough windows of 8 W residues for every resident CTA
  // (up to two per SM) to scan two, so each candidate shape is timed on a full grid
  if (sample_len <= 0) sample_len = std::max<int64_t>((int64_t) c->nsm * 1500, (int64_t) c->nsm * 4 * 8 * m->W);
  std::vector<uint8_t> dsq((size_t) sample_len + 2);
  uint64_t x = 0x9E3779B97F4A7C15ULL;
  for (int64_t i = 1; i <= sample_len; i++) {            // 40% GC, splitmix-style generator
    x += 0x9E3779B97F4A7C15ULL; uint64_t z = x; z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL; z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL; z ^= z >> 31;
    const unsigned u = (unsigned) (z % 100);
    dsq[i] = u < 30 ? 0 : u < 50 ? 1 : u < 70 ? 2 : 3;
  }
  dsq[0] = dsq[sample_len + 1] = 255;
  static const int cand[][2] = {{16, 1}, {32, 2}, {48, 2}, {64, 2}, {96, 2}, {128, 2}};
  const int saveT = c->tile_rows, saveA = c->arena;
  float best_ms = 3.0e38f; int bT = 16, bA = 1;
  int st = CMGB_OK;
  for (const auto &cd : cand) {
    c->tile_rows = cd[0]; c->arena = cd[1];
    float ms = 0.f;
    for (int rep = 0; rep < 2 && st == CMGB_OK; rep++) {   // first run builds the plan and warms up
      st = scan_std(c, m, errbuf, qdbidx, algo, dsq.data(), nullptr, 1, sample_len, 1e30f, nullptr, 0, 1e30f, nullptr, nullptr, nullptr, nullptr);
      ms = c->last_ms;
    }
    if (st != CMGB_OK) {           // a shape that does not fit this device is skipped
      if (st == CMGB_ENODEV) break;
      st = CMGB_OK;
      continue;
    }
    if (ms < best_ms) { best_ms = ms; bT = cd[0]; bA = cd[1]; }
  }
  c->tile_rows = saveT; c->arena = saveA;
  if (st != CMGB_OK) return st;
  m->tuned_T[qdbidx][algo] = bT; m->tuned_arena[qdbidx][algo] = bA;
  if (ret_tile_rows) *ret_tile_rows = bT;
  if (ret_arena) *ret_arena = bA;
  return CMGB_OK;
}

extern "C" int64_t cmgb_count_cells(const cmgb_model_desc *m, int qdbidx, int64_t L)
{
  const int *dmin = qdbidx == 1 ? m->dmin1 : qdbidx == 2 ? m->dmin2 : nullptr;
  const int *dmax = qdbidx == 1 ? m->dmax1 : qdbidx == 2 ? m->dmax2 : nullptr;
  const int Wl = (int) (m->W > L ? L : m->W);
  int64_t cells = 0;
  for (int v = 0; v < m->M; v++) {
    if (m->sttype[v] == CMGB_E_st) continue;
    int lo = m->sttype[v] == CMGB_MP_st ? 2 : 1;
    if (dmin) lo = std::max(dmin[v], lo);
    const int dn = std::min(lo, m->W), dx = dmax ? std::min(dmax[v], m->W) : m->W;
    for (int64_t jp = 1; jp <= L && jp < Wl; jp++) { int hi = std::min((int) jp, dx); if (hi >= dn) cells += hi - dn + 1; }
    if (L >= Wl) { int hi = std::min(Wl, dx); if (hi >= dn) cells += (int64_t) (hi - dn + 1) * (L - Wl + 1); }
  }
  return cells;
}

// ---------------------------------------------------------------------------
// Allocation-free CYK scan (cmgb_FastCYKScan_noalloc): scratch in a static
// device array, outputs in caller-provided device memory.
#ifndef CMGB_HOST_EMULATION
static __device__ __align__(256) unsigned char g_noalloc_scratch[CMGB_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch on each device, looked up once per device.
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64];

static __global__ void noalloc_init_kernel(int *queue, Control *ctl)
{
  *queue = 0;
  ctl->queue = 0; ctl->ncand = 0; ctl->err = 0;
  ctl->env[0] = LLONG_MAX; ctl->env[1] = -1;
  ctl->best = 0u;
}

static int noalloc_scan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx,
                        const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff, float env_cutoff,
                        cmgb_cell *d_cells, int cell_cap, int *ret_ncells,
                        int64_t *ret_envi, int64_t *ret_envj, float *ret_sc);
#endif

extern "C" int cmgb_FastCYKScan_noalloc(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx,
                                        const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff, float env_cutoff,
                                        cmgb_cell *d_cells, int cell_cap, int *ret_ncells,
                                        int64_t *ret_envi, int64_t *ret_envj, float *ret_sc)
{
#ifdef CMGB_HOST_EMULATION
  (void) c; (void) m; (void) qdbidx; (void) d_dsq; (void) i0; (void) j0; (void) cutoff; (void) env_cutoff;
  (void) d_cells; (void) cell_cap; (void) ret_ncells; (void) ret_envi; (void) ret_envj; (void) ret_sc;
  ERRF(CMGB_ENODEV, "FastCYKScan_noalloc, not available in the host emulation");
#else
  // the scan runs with the context's device current; the caller's current device is restored on every return
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  const int st = noalloc_scan(c, m, errbuf, qdbidx, d_dsq, i0, j0, cutoff, env_cutoff, d_cells, cell_cap, ret_ncells,
                              ret_envi, ret_envj, ret_sc);
  if (prev >= 0) cudaSetDevice(prev);
  return st;
#endif
}

#ifndef CMGB_HOST_EMULATION
static int noalloc_scan(cmgb_ctx *c, cmgb_model *m, char *errbuf, int qdbidx,
                        const uint8_t *d_dsq, int64_t i0, int64_t j0, float cutoff, float env_cutoff,
                        cmgb_cell *d_cells, int cell_cap, int *ret_ncells,
                        int64_t *ret_envi, int64_t *ret_envj, float *ret_sc)
{
  if (!c || !m) ERRF(CMGB_EINVAL, "FastCYKScan_noalloc, NULL context or model");
  if (j0 < i0 || i0 < 1) ERRF(CMGB_EINCOMPAT, "FastCYKScan_noalloc, i0: %lld j0: %lld", (long long) i0, (long long) j0);
  if (d_dsq == nullptr) ERRF(CMGB_EINCOMPAT, "FastCYKScan_noalloc, dsq is NULL");
  if (qdbidx < 0 || qdbidx > 2) ERRF(CMGB_EINCOMPAT, "FastCYKScan_noalloc, qdbidx is invalid");
  if (d_cells == nullptr || cell_cap <= 0) ERRF(CMGB_EINVAL, "FastCYKScan_noalloc, no output cell array");
  if (c->device < 0 || c->device >= 64) ERRF(CMGB_ENODEV, "FastCYKScan_noalloc, device index out of range");
  CUDA_TRY(cudaSetDevice(c->device));
  void *scratch;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[c->device]) {
      void *ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) ERRF(CMGB_ENODEV, "FastCYKScan_noalloc, cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      g_noalloc_ptr[c->device] = ptr;
    }
    scratch = g_noalloc_ptr[c->device];
  }
  const DevPlan &dp = m->plans[qdbidx][0];
  if (!dp.built) ERRF(CMGB_EINCOMPAT, "FastCYKScan_noalloc, no plan for band set %d yet: run a scan on this context first", qdbidx);
  const ScanPlan &P = dp.plan;
  const bool gl = P.arena_global != 0;
  const int64_t L = j0 - i0 + 1;

  // scratch layout (256-byte aligned regions): work counter, control block, then per CTA
  // carry rows (two parities), BEGL ring and, for global-arena plans, the tile arena
  auto al = [](size_t x) { return (x + 255) & ~(size_t) 255; };
  const size_t per_cta = al(sizeof(float) * 2 * (size_t) P.carry_elems) + al(sizeof(float) * (size_t) P.ring_elems) +
                         (gl ? al(sizeof(float) * (size_t) P.arena_elems) : 0);
  const size_t head = 256 + al(sizeof(Control));
  if (head + per_cta + 1024 > (size_t) CMGB_NOALLOC_SCRATCH_BYTES)
    ERRF(CMGB_ERANGE, "FastCYKScan_noalloc, the model needs %zu bytes of scratch per CTA; the static array holds %u",
         per_cta, (unsigned) CMGB_NOALLOC_SCRATCH_BYTES);
  int nb = 1;
  if (gl) CUDA_TRY((prepare_qdb<false, true>(c->threads, P.smem_bytes, &nb)));
  else    CUDA_TRY((prepare_qdb<false, false>(c->threads, P.smem_bytes, &nb)));
  const int cps = c->ctas_per_sm > 0 ? c->ctas_per_sm : (nb < 1 ? 1 : nb);
  int64_t grid_max = (int64_t) c->nsm * cps;
  const int64_t fit = (int64_t) (((size_t) CMGB_NOALLOC_SCRATCH_BYTES - head - 1024) / per_cta);   // 1024: room for region alignment
  if (grid_max > fit) grid_max = fit;
  int64_t win = c->window_len;
  if (win <= 0) {
    win = (L + grid_max - 1) / grid_max;
    if (win < 8LL * m->W) win = 8LL * m->W;
  }
  win = ((win + P.T - 1) / P.T) * P.T;
  const int64_t nwin = (L + win - 1) / win;
  if (nwin > INT_MAX) ERRF(CMGB_ERANGE, "FastCYKScan_noalloc, too many windows");
  const int grid = (int) std::min<int64_t>(nwin, grid_max);

  unsigned char *base = (unsigned char *) scratch;
  int *queue = (int *) base;
  Control *ctl = (Control *) (base + 256);
  unsigned char *cta0 = base + head;
  // carry, ring and arena are laid out as [grid][...] arrays, as the kernel indexes them
  float *carry = (float *) cta0;
  float *ring = (float *) (cta0 + al(sizeof(float) * 2 * (size_t) P.carry_elems * grid));
  float *arena = (float *) ((unsigned char *) ring + al(sizeof(float) * (size_t) P.ring_elems * grid));
  if ((size_t) ((unsigned char *) arena - base) + (gl ? sizeof(float) * (size_t) P.arena_elems * grid : 0) > (size_t) CMGB_NOALLOC_SCRATCH_BYTES)
    ERRF(CMGB_ERANGE, "FastCYKScan_noalloc, scratch layout exceeds the static array");

  noalloc_init_kernel<<<1, 1, 0, c->stream>>>(queue, ctl);
  CUDA_TRY(cudaGetLastError());
  KParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.st = dp.d_states; kp.plan = P; kp.rec = dp.d_rec; kp.arena = gl ? arena : nullptr;
  kp.oesc = m->d_oesc; kp.ioesc = m->d_ioesc; kp.ilog = c->d_ilog;
  kp.dsq = d_dsq; kp.i0 = i0; kp.j0 = j0; kp.win_len = win; kp.nwin = (int) nwin;
  kp.queue = queue; kp.carry = carry; kp.ring = ring;
  kp.cand = reinterpret_cast<Cand *>(d_cells); kp.ncand = &ctl->ncand; kp.cand_cap = cell_cap;
  // the candidate set of cmgb_FastCYKScan: cells >= cutoff (greedy), cells > 0 (optimal resolution)
  kp.cand_cut = cutoff; kp.cand_pos = (m->flags & CMGB_NOTGREEDY) ? 1 : 0;
  kp.env_cut = env_cutoff; kp.env = ctl->env; kp.vsc = nullptr; kp.best = &ctl->best; kp.err = &ctl->err;
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  if (gl) launch_qdb<false, true>(grid, c->threads, (size_t) P.smem_bytes, c->stream, kp);
  else    launch_qdb<false, false>(grid, c->threads, (size_t) P.smem_bytes, c->stream, kp);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  Control h;
  CUDA_TRY(cudaMemcpyAsync(&h, ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  c->last_launches = 2;
  if (h.err & 2) ERRF(CMGB_ENODEV, "FastCYKScan_noalloc, a bounded device wait ran out (phase record copy)");
  if (h.err & 1) ERRF(CMGB_ERANGE, "FastCYKScan_noalloc, more than %d candidate cells", cell_cap);
  if (ret_ncells) *ret_ncells = h.ncand;
  if (ret_envi) *ret_envi = (h.env[1] < 0) ? -1 : h.env[0];
  if (ret_envj) *ret_envj = (h.env[1] < 0) ? -1 : h.env[1];
  if (ret_sc) {
    const unsigned u = h.best;
    float f = CMGB_IMPOSSIBLE;
    if (u != 0) { unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u; std::memcpy(&f, &b, 4); }
    *ret_sc = f;
  }
  return CMGB_OK;
}
#endif

// ---------------------------------------------------------------------------
// Measured issue peaks of the DP's arithmetic: the roofline denominators of
// the scan kernels.  Every thread runs 8 independent chains of
// x = max(x + y, z) -- one add and one max, the CYK fold's pair of
// operations (kind 0: fp32 round-to-nearest add and fmaxf) or the integer
// Inside's (kind 1: int32 add and max) -- on every SM at 2048 threads per SM.
#ifndef CMGB_HOST_EMULATION
template <int KIND>
static __global__ void __launch_bounds__(256) issue_peak_kernel(const int *in, int *out, int iters)
{
  if (KIND == 0) {
    const float y = __int_as_float(in[0]), z = __int_as_float(in[1]);
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (float) (threadIdx.x + k);
#pragma unroll 4
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = fmaxf(__fadd_rn(x[k], y), z);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s = __fadd_rn(s, x[k]);
    if (in[2]) out[blockIdx.x * blockDim.x + threadIdx.x] = __float_as_int(s);
  } else {
    const int y = in[0], z = in[1];
    int x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (int) threadIdx.x + k;
#pragma unroll 4
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = max(x[k] + y, z);
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (in[2]) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  }
}
#endif

extern "C" int cmgb_measure_issue_peak(cmgb_ctx *c, int kind, double *ret_ops_per_s, char *errbuf)
{
#ifdef CMGB_HOST_EMULATION
  (void) c; (void) kind; (void) ret_ops_per_s;
  ERRF(CMGB_ENODEV, "measure_issue_peak, not available in the host emulation");
#else
  if (!c || !ret_ops_per_s || kind < 0 || kind > 1) ERRF(CMGB_EINVAL, "measure_issue_peak, invalid arguments");
  CUDA_TRY(cudaSetDevice(c->device));
  const int threads = 256, blocks = c->nsm * 8, iters = 1 << 16;
  int *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(int) * (4 + (size_t) blocks * threads)));
  // y = -1, z = a large negative floor, no output (in[2] = 0)
  const float fy = -1.0f, fz = -1.0e30f;
  int h[4] = {0, 0, 0, 0};
  if (kind == 0) { std::memcpy(&h[0], &fy, 4); std::memcpy(&h[1], &fz, 4); }
  else { h[0] = -1; h[1] = -1000000000; }
  cudaError_t e = cudaMemcpy(d, h, sizeof(h), cudaMemcpyHostToDevice);
  float best = 1e30f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
    cudaEventRecord(c->ev0, c->stream);
    if (kind == 0) issue_peak_kernel<0><<<blocks, threads, 0, c->stream>>>(d, d + 4, iters);
    else           issue_peak_kernel<1><<<blocks, threads, 0, c->stream>>>(d, d + 4, iters);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    cudaEventRecord(c->ev1, c->stream);
    e = cudaEventSynchronize(c->ev1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (rep > 0 && ms < best) best = ms;      // rep 0 warms up
  }
  cudaFree(d);
  if (e != cudaSuccess) ERRF(CMGB_ENODEV, "measure_issue_peak: %s", cudaGetErrorString(e));
  *ret_ops_per_s = 2.0 * 8.0 * (double) iters * (double) blocks * threads / (best * 1e-3);
  return CMGB_OK;
#endif
}
