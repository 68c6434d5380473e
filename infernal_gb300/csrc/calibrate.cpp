// calibrate.cpp -- E-value calibration of a model on the GPU: the procedure
// of the reference's cmcalibrate (src/cmcalibrate.c) for one search mode,
// built on the batched scanner (cmgb_ScanBatch).
//
// The reference generates N random sequences of length L (dbsize = N * L,
// 1.6 Mb by default), scans them with FastCYKScan or FastIInsideScan at the
// QDB2 bands (process_search_workunit, :2328-2370), adds every hit score to a
// histogram and fits an exponential to the best --ltailn / --gtailn hits per
// Mb (fit_histogram, :1930-2020; esl_exp_FitComplete).  Here the random
// sequence is a project-defined background (segments of geometric length,
// mean 2.5 kb, each at a GC content drawn uniformly from 0.30-0.65) from a
// seeded splitmix64 stream; all pieces are scanned in one batched launch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/infernal_gb300.h"

#define CERR(code, ...) do { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, __VA_ARGS__); return (code); } while (0)

namespace {
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double) (next() >> 11) * (1.0 / 9007199254740992.0); }
};

// One random piece: Easel digital codes 0..3 (A C G U) between sentinels.
void background_piece(SplitMix &rng, int64_t n, uint8_t *out)
{
  out[0] = 255;
  double gc = 0.30 + 0.35 * rng.uniform();
  for (int64_t i = 1; i <= n; i++) {
    if (rng.uniform() < 1.0 / 2500.0) gc = 0.30 + 0.35 * rng.uniform();   // segment boundary
    const double u = rng.uniform();
    const double at = 0.5 * (1.0 - gc), g2 = 0.5 * gc;
    out[i] = u < at ? 0 : u < at + g2 ? 1 : u < at + 2 * g2 ? 2 : 3;
  }
  out[n + 1] = 255;
}
}  // namespace

extern "C" int cmgb_Calibrate(cmgb_ctx *c, cmgb_model *m, char *errbuf, int algo, int64_t total_len, int64_t seq_len,
                              uint64_t seed, int tail_per_mb, cmgb_expinfo *ret, float *ret_ms)
{
  if (!c || !m || !ret) CERR(CMGB_EINVAL, "Calibrate, NULL context, model or result");
  if (algo != CMGB_ALGO_CYK && algo != CMGB_ALGO_IINSIDE) CERR(CMGB_EINVAL, "Calibrate, algorithm %d is not CYK or integer Inside", algo);
  if (total_len < 1000 || seq_len < 100 || tail_per_mb < 1) CERR(CMGB_EINVAL, "Calibrate, invalid sizes");
  const int64_t ntail = (int64_t) std::llround((double) tail_per_mb * (double) total_len / 1e6);
  if (ntail < 2) CERR(CMGB_ERANGE, "Calibrate, a tail of %lld hits is too small to fit", (long long) ntail);

  // the random database: pieces of seq_len residues (the last one shorter)
  const int nseq = (int) ((total_len + seq_len - 1) / seq_len);
  std::vector<int64_t> offsets(nseq), lengths(nseq);
  std::vector<uint8_t> buf;
  buf.reserve((size_t) (total_len + 2 * nseq + 1));
  SplitMix rng{seed ^ 0x5DEECE66DULL};
  for (int q = 0; q < nseq; q++) {
    const int64_t n = std::min<int64_t>(seq_len, total_len - (int64_t) q * seq_len);
    offsets[q] = (int64_t) buf.size();
    lengths[q] = n;
    buf.resize(buf.size() + (size_t) n + 2);
    background_piece(rng, n, buf.data() + offsets[q]);
  }
  buf.push_back(255);

  // scan at a cutoff below the tail; lower it until the tail is collected
  // in 15-bit steps (hits above a cutoff do not depend on it: greedy
  // resolution takes the best scores first)
  cmgb_hitlist *hl = cmgb_hitlist_create();
  std::vector<float> sc;
  float ms_tot = 0.f;
  int st = CMGB_OK;
  for (float cut = 0.0f; cut >= -120.0f; cut -= 15.0f) {   // glocal tails can start near -45 bits
    cmgb_hitlist_clear(hl);
    st = cmgb_ScanBatch(c, m, errbuf, algo, CMGB_QDB2_LOOSE, 0, buf.data(), (int64_t) buf.size(), offsets.data(),
                        lengths.data(), nseq, cut, hl, 1, cut, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (st != CMGB_OK) break;
    ms_tot += cmgb_ctx_last_kernel_ms(c);
    sc.clear();
    cmgb_hit h;
    for (int64_t k = 0; k < cmgb_hitlist_count(hl); k++) { cmgb_hitlist_get(hl, k, &h); sc.push_back(h.score); }
    if ((int64_t) sc.size() >= ntail) break;
  }
  cmgb_hitlist_destroy(hl);
  if (st != CMGB_OK) return st;
  if ((int64_t) sc.size() < ntail)
    CERR(CMGB_ERANGE, "Calibrate, only %zu hits down to -120 bits; the tail needs %lld", sc.size(), (long long) ntail);

  // maximum-likelihood exponential with known origin over the best ntail scores
  std::sort(sc.begin(), sc.end(), [](float a, float b) { return a > b; });
  const double mu = (double) sc[(size_t) ntail - 1];
  double sum = 0.0;
  for (int64_t k = 0; k < ntail; k++) sum += (double) sc[(size_t) k] - mu;
  const double mean = sum / (double) ntail;
  if (!(mean > 0.0)) CERR(CMGB_ERANGE, "Calibrate, degenerate tail (all %lld scores equal)", (long long) ntail);
  ret->lambda = 1.0 / mean;
  ret->mu_orig = mu;
  ret->mu_extrap = mu;   // tailp = 1: mu_orig - log(1 / tailp) / lambda
  ret->dbsize = (double) total_len;
  ret->nrandhits = ntail;
  ret->tailp = 1.0;
  if (ret_ms) *ret_ms = ms_tot;
  return CMGB_OK;
}
