// hits.h -- host-side hit resolution for the GB300 scanners.
//
// The kernels emit every root cell (j, d) that can become a hit: score >=
// cutoff for greedy resolution (a NULL3 correction only lowers a score), or
// score > 0 for optimal resolution.  This file turns those candidates into
// the reference's hit list:
//   greedy  : ReportHitsGreedily          src/cm_mx.c:7547-7628
//             then SortForOverlapRemoval + RemoveOrMarkOverlaps
//             src/cm_tophits.c:220-245, 400, 1097-1275
//   optimal : UpdateGammaHitMx / TBackGammaHitMx src/cm_mx.c:7440-7669
//   NULL3   : ScoreCorrectionNull3        src/cm_parsetree.c:2352-2380
// Cells absent from the candidate list could never pass the reference's
// tests, so the result is identical to resolving every cell.
#pragma once
#include <stdint.h>
#include <functional>
#include <vector>
#include "../../include/infernal_gb300.h"

namespace cmgb {

// A resolved root cell: end j, length d, score, root state, mode (standard
// scans: CMGB_TRMODE_J).
struct CandHost { long long j; int d; float sc; int r; int mode; };

// Truncated scans: which hits a pass may report, cm_hit_AllowTruncation
// (src/cm_tophits.c:3048-3090).
struct TruncFilter {
  int pass_idx;
  int local;             // CMH_LOCAL_BEGIN
  int clen;
  const int *ndidx;      // [M]
  const int8_t *ndtype;  // [nodes]
  const int *lpos, *rpos;// emit map [nodes]
};
bool allow_truncation(const TruncFilter &t, int64_t start, int64_t stop, int64_t i0, int64_t j0, int mode, int b);

// f(0) .. f(n-1) on up to 16 host threads (the resolution of independent
// sequences of a batch)
void parallel_for(int n, const std::function<void(int)> &f);

struct ResolveArgs {
  const float *null;     // [K]
  int K;
  float null3_omega;
  int do_null3;
  int greedy;            // 1: greedy, 0: optimal (gamma)
  float cutoff;
  int64_t i0, j0;
  const uint8_t *dsq;    // host residues indexed by sequence coordinate (needed for NULL3)
  const TruncFilter *tr = nullptr;   // truncated scans: per-hit admissibility and modes
};

// Appends the resolved hits to out (in the reference's order).
void resolve_hits(std::vector<CandHost> &cands, const ResolveArgs &a, std::vector<cmgb_hit> &out);

// LogSum2 table init (FLogsumInit, src/logsum.c:138) and integer ILogsum table (src/logsum.c:74).
void logsum_tables(const float **flog, const int **ilog);

}  // namespace cmgb
