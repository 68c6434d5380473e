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
#include <vector>
#include "../../include/infernal_gb300.h"

namespace cmgb {

struct CandHost { long long j; int d; float sc; int r; int pad; };

struct ResolveArgs {
  const float *null;     // [K]
  int K;
  float null3_omega;
  int do_null3;
  int greedy;            // 1: greedy, 0: optimal (gamma)
  float cutoff;
  int64_t i0, j0;
  const uint8_t *dsq;    // host residues indexed by sequence coordinate (needed for NULL3)
};

// Appends the resolved hits to out (in the reference's order).
void resolve_hits(std::vector<CandHost> &cands, const ResolveArgs &a, std::vector<cmgb_hit> &out);

// LogSum2 table init (FLogsumInit, src/logsum.c:138) and integer ILogsum table (src/logsum.c:74).
void logsum_tables(const float **flog, const int **ilog);

}  // namespace cmgb
