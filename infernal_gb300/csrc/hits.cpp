// hits.cpp -- host-side hit resolution (see hits.h for the reference map).
#include "hits.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>

namespace cmgb {

static const float IMPf = -1e36f;
static inline bool not_imp(float x) { return x > -9.999e35f; }
static inline double log2d(double x) { return x > 0 ? std::log(x) * 1.44269504 : -1e36; }  // sreLOG2

static float flog_tbl[23000];
static int ilog_tbl[23000];
static std::once_flag tables_once;

void logsum_tables(const float **flog, const int **ilog)
{
  std::call_once(tables_once, [] {
    for (int i = 0; i < 23000; i++) {
      double x = log2d(1. + std::exp(((double) -i / 1000.0f) * 0.69314718));
      flog_tbl[i] = (float) x;
      ilog_tbl[i] = (int) std::rint(1000.0f * x);
    }
  });
  if (flog) *flog = flog_tbl;
  if (ilog) *ilog = ilog_tbl;
}

void parallel_for(int n, const std::function<void(int)> &f)
{
  const int nt = std::min<int>(n, std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
  if (nt <= 1) { for (int i = 0; i < n; i++) f(i); return; }
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++)
    th.emplace_back([&] { for (int i; (i = next.fetch_add(1)) < n;) f(i); });
  for (auto &x : th) x.join();
}

// Candidates in (j, d) order.  The cells are distinct, so two stable
// counting passes (by d, then by j) give the order a comparison sort gives;
// they are used when the j range is not much wider than the candidate count.
static void sort_jd(std::vector<CandHost> &c)
{
  if (c.size() < 2) return;
  long long jmin = c[0].j, jmax = c[0].j;
  int dmax = 0;
  for (const CandHost &x : c) { jmin = std::min(jmin, x.j); jmax = std::max(jmax, x.j); dmax = std::max(dmax, x.d); }
  const long long range = jmax - jmin + 1;
  if (c.size() < 2048 || range > 8 * (long long) c.size()) {
    std::sort(c.begin(), c.end(), [](const CandHost &x, const CandHost &y) { return x.j != y.j ? x.j < y.j : x.d < y.d; });
    return;
  }
  std::vector<CandHost> tmp(c.size());
  std::vector<int64_t> cnt((size_t) dmax + 2, 0);
  for (const CandHost &x : c) cnt[(size_t) x.d + 1]++;
  for (size_t k = 1; k < cnt.size(); k++) cnt[k] += cnt[k - 1];
  for (const CandHost &x : c) tmp[(size_t) cnt[(size_t) x.d]++] = x;
  std::vector<int64_t> cj((size_t) range + 1, 0);
  for (const CandHost &x : tmp) cj[(size_t) (x.j - jmin) + 1]++;
  for (size_t k = 1; k < cj.size(); k++) cj[k] += cj[k - 1];
  for (const CandHost &x : tmp) c[(size_t) cj[(size_t) (x.j - jmin)]++] = x;
}

// LogSum2 / FLogsum (src/logsum.c:151-168)
static inline float logsum2(float s1, float s2)
{
  const float mx = s1 > s2 ? s1 : s2, mn = s1 < s2 ? s1 : s2;
  return (mn == -INFINITY || (mx - mn) >= 23.f) ? mx : mx + flog_tbl[(int) ((mx - mn) * 1000.0f)];
}

// Residue weights of the RNA alphabet: canonical codes count 1, degenerate
// codes spread 1 evenly over the residues they stand for.
static const uint8_t degen_mask[18] = {1, 2, 4, 8, 0, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 0, 0};
static inline void count_res(double *ct, uint8_t x, int K)
{
  if (x < K) { ct[x] += 1.; return; }
  if (x >= 18) return;
  int n = __builtin_popcount(degen_mask[x]);
  if (!n) return;
  for (int y = 0; y < K; y++) if (degen_mask[x] & (1 << y)) ct[y] += 1. / (double) n;
}

// Exact residue composition of [i, j]: the reference differences two running
// sums that start at i0 (act[], src/cm_dpsearch.c:199-231).  When every code
// in the range has weight 1, 1/2 or 1/4 those sums are exact, and so are
// integer prefix counts in quarter units, which give the same doubles in
// O(1) per lookup (ranges longer than kPrefixMaxResidues count each lookup's
// residues instead, the same doubles without 16 bytes per residue).
// Three-way codes (H, B, V, D) need the running doubles themselves: they are
// accumulated in order from i0 as lookups ask for later end positions (the
// resolvers visit end positions in increasing order), and a ring keeps the
// last maxd + 1 rows, as the reference's act[jp % (W+1)].
static const int64_t kPrefixMaxResidues = 16 << 20;
struct Composition {
  const uint8_t *dsq; int64_t i0, j0; int K;
  bool exact_direct = true;
  bool counted = false;          // exact_direct over a range too long for prefix counts: count per lookup
  std::vector<int32_t> qprefix;  // (j0-i0+2) x K running counts in quarter units (exact_direct)
  // three-way codes: running sums of positions i0-1 .. cur in a ring of R rows
  int R = 0;
  mutable int64_t cur = 0;
  mutable std::vector<double> ring;
  Composition(const uint8_t *q, int64_t a, int64_t b, int k, int maxd) : dsq(q), i0(a), j0(b), K(k) {
    for (int64_t x = i0; x <= j0; x++) { uint8_t c = dsq[x]; if (c >= K && c < 18 && __builtin_popcount(degen_mask[c]) == 3) { exact_direct = false; break; } }
    if (!exact_direct) {
      R = maxd + 2;
      ring.assign((size_t) R * K, 0.);   // row of position i0-1: all zero
      cur = i0 - 1;
      return;
    }
    if (j0 - i0 + 1 > kPrefixMaxResidues) { counted = true; return; }
    qprefix.assign((size_t) (j0 - i0 + 2) * K, 0);
    for (int64_t x = i0; x <= j0; x++) {
      int32_t *row = &qprefix[(size_t) (x - i0 + 1) * K];
      std::memcpy(row, row - K, sizeof(int32_t) * K);
      const uint8_t c = dsq[x];
      if (c < K) row[c] += 4;
      else if (c < 18) {
        const int nb = __builtin_popcount(degen_mask[c]);
        if (nb) for (int y = 0; y < K; y++) if (degen_mask[c] & (1 << y)) row[y] += 4 / nb;
      }
    }
  }
  const double *ring_row(int64_t x) const { return &ring[(size_t) ((x - i0 + 1) % R) * K]; }
  void get(int64_t i, int64_t j, float *comp) const {
    if (counted) {
      double ct[8] = {0};
      for (int64_t x = i; x <= j; x++) count_res(ct, dsq[x], K);
      for (int a = 0; a < K; a++) comp[a] = (float) ct[a];
    } else if (exact_direct) {
      const int32_t *hi = &qprefix[(size_t) (j - i0 + 1) * K], *lo = &qprefix[(size_t) (i - i0) * K];
      for (int a = 0; a < K; a++) comp[a] = (float) ((double) (hi[a] - lo[a]) * 0.25);
    } else {
      while (cur < j) {   // accumulate the running sums up to j
        const double *prev = ring_row(cur);
        cur++;
        double *row = const_cast<double *>(ring_row(cur));
        if (row != prev) std::memcpy(row, prev, sizeof(double) * K);
        count_res(row, dsq[cur], K);
      }
      const double *hi = ring_row(j), *lo = ring_row(i - 1);
      for (int a = 0; a < K; a++) comp[a] = (float) (hi[a] - lo[a]);
    }
  }
};

static float fsum_kahan(const float *v, int n)
{
  float s = 0.f, c = 0.f, y, t;
  for (int i = 0; i < n; i++) { y = v[i] - c; t = s + y; c = (t - s) - y; s = t; }
  return s;
}

// ScoreCorrectionNull3 (src/cm_parsetree.c:2352) after esl_vec_FNorm of comp
static float null3(const ResolveArgs &a, const Composition &cmp, int64_t i, int64_t j)
{
  float comp[8];
  cmp.get(i, j, comp);
  float s = fsum_kahan(comp, a.K);
  if (s != 0.f) for (int x = 0; x < a.K; x++) comp[x] /= s;
  else          for (int x = 0; x < a.K; x++) comp[x] = 1.f / (float) a.K;
  const int len = (int) (j - i + 1);
  float score = 0.f;
  for (int x = 0; x < a.K; x++) score += log2d(comp[x] / a.null[x]) * comp[x] * len;
  score += log2d(a.null3_omega);
  return logsum2(0.f, score);
}

bool allow_truncation(const TruncFilter &t, int64_t start, int64_t stop, int64_t i0, int64_t j0, int mode, int b)
{
  const int nd = t.ndidx[b], nt = t.ndtype[nd];
  const int lpos = (nt == CMGB_MATP_nd || nt == CMGB_MATL_nd) ? t.lpos[nd] : t.lpos[nd] + 1;
  const int rpos = (nt == CMGB_MATP_nd || nt == CMGB_MATR_nd) ? t.rpos[nd] : t.rpos[nd] - 1;
  if (t.pass_idx == CMGB_PASS_STD_ANY || t.pass_idx == CMGB_PASS_5P_AND_3P_ANY || t.pass_idx == CMGB_PASS_HMM_ONLY_ANY) return true;
  if (start == i0 && stop == j0) return true;
  if (t.local) {
    switch (mode) {
    case CMGB_TRMODE_J: return true;
    case CMGB_TRMODE_L: return stop == j0;
    case CMGB_TRMODE_R: return start == i0;
    default: return false;
    }
  }
  switch (mode) {
  case CMGB_TRMODE_J: return lpos == 1 && rpos == t.clen;
  case CMGB_TRMODE_L: return stop == j0 && lpos == 1;
  case CMGB_TRMODE_R: return start == i0 && rpos == t.clen;
  default: return false;
  }
}

void resolve_hits(std::vector<CandHost> &c, const ResolveArgs &a, std::vector<cmgb_hit> &out)
{
  logsum_tables(nullptr, nullptr);
  sort_jd(c);
  Composition *cmp = nullptr;
  if (a.do_null3 && !c.empty()) {
    int maxd = 1;
    for (const CandHost &x : c) maxd = std::max(maxd, x.d);
    cmp = new Composition(a.dsq, a.i0, a.j0, a.K, maxd);
  }

  if (a.greedy) {
    // ReportHitsGreedily per j, then greedy overlap removal
    std::vector<cmgb_hit> tmp;
    size_t k = 0;
    while (k < c.size()) {
      size_t e = k;
      while (e < c.size() && c[e].j == c[k].j) e++;
      float best = IMPf;
      for (size_t q = k; q < e; q++) {
        float hs = c[q].sc;
        if (hs > best && hs >= a.cutoff && not_imp(hs)) {
          bool rep = true;
          int64_t i = c[q].j - c[q].d + 1;
          const int mode = a.tr ? c[q].mode : CMGB_TRMODE_J;
          if (a.tr) rep = allow_truncation(*a.tr, i, c[q].j, a.i0, a.j0, mode, c[q].r);
          if (rep && cmp) { hs -= null3(a, *cmp, i, c[q].j); rep = (hs > best && hs >= a.cutoff); }
          if (rep) { cmgb_hit h; h.start = i; h.stop = c[q].j; h.root = c[q].r; h.mode = mode; h.score = hs; tmp.push_back(h); best = hs; }
        }
      }
      k = e;
    }
    // sort: score high to low, then start low to high (src/cm_tophits.c:220-245);
    // ties beyond that keep creation order
    std::stable_sort(tmp.begin(), tmp.end(), [](const cmgb_hit &x, const cmgb_hit &y) {
      if (x.score != y.score) return x.score > y.score;
      return x.start < y.start;
    });
    // keep a hit only if it overlaps no better hit already kept
    std::map<int64_t, int64_t> kept;   // start -> stop of kept hits (disjoint)
    for (const cmgb_hit &h : tmp) {
      auto it = kept.upper_bound(h.stop);   // first kept start > h.stop
      bool overlap = false;
      if (it != kept.begin()) { auto pr = std::prev(it); if (pr->second >= h.start) overlap = true; }
      if (!overlap) { kept[h.start] = h.stop; out.push_back(h); }
    }
  } else {
    // optimal resolution: gamma semi-HMM over end positions
    const int64_t L = a.j0 - a.i0 + 1;
    std::vector<float> mx(L + 1);
    std::vector<int64_t> gback(L + 1, -1);
    std::vector<float> savesc(L + 1, IMPf);
    std::vector<int> saver(L + 1, -1), savemode(L + 1, -1);
    mx[0] = 0.f;
    size_t k = 0;
    for (int64_t jp = 1; jp <= L; jp++) {
      const int64_t j = a.i0 + jp - 1;
      mx[jp] = mx[jp - 1];
      while (k < c.size() && c[k].j < j) k++;
      while (k < c.size() && c[k].j == j) {
        const int d = c[k].d;
        const int64_t ip = jp - d + 1;
        float hs = c[k].sc, cum = mx[ip - 1] + hs;
        if (cum > mx[jp] && not_imp(hs)) {
          bool rep = true;
          const int mode = a.tr ? c[k].mode : CMGB_TRMODE_J;
          if (a.tr) rep = allow_truncation(*a.tr, j - d + 1, j, a.i0, a.j0, mode, c[k].r);
          if (rep && cmp) { float c3 = null3(a, *cmp, j - d + 1, j); hs -= c3; cum -= c3; rep = cum > mx[jp]; }
          if (rep) { mx[jp] = cum; gback[jp] = j - d + 1; savesc[jp] = hs; saver[jp] = c[k].r; savemode[jp] = mode; }
        }
        k++;
      }
    }
    int64_t j = a.j0;
    while (j >= a.i0) {
      const int64_t jp = j - a.i0 + 1;
      if (gback[jp] == -1) j--;
      else {
        if (savesc[jp] >= a.cutoff) { cmgb_hit h; h.start = gback[jp]; h.stop = j; h.root = saver[jp]; h.mode = savemode[jp]; h.score = savesc[jp]; out.push_back(h); }
        j = gback[jp] - 1;
      }
    }
  }
  delete cmp;
}

}  // namespace cmgb
