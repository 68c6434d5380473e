// scan_plan.h -- per-(model, band set) execution plan of the tiled QDB scan.
//
// The GPU scan advances each sequence window in tiles of T end positions j.
// Inside a tile the states are swept from v = M-1 down to 0 (children before
// parents, the order of the reference's `for (v = cm->M-1; ...)` loop,
// src/cm_dpsearch.c:233), and every state's T x band cells are computed at
// once from its children's tiles, which sit in shared memory.  A state's tile
// buffer holds rows r = 0..T: row 0 is the state's last row of the previous
// tile (the "carry", kept in global memory between tiles), rows 1..T are
// j = t .. t+T-1.  Each buffer covers the padded d-range [lo, hi]: the
// state's own band plus every cell any parent reads; cells outside the
// state's band hold the values the reference's scan matrix holds there
// (its d = 0 initialisation, src/cm_mx.c:6039-6082, or IMPOSSIBLE), so the
// recurrences read children without per-cell band tests.
//
// This header is shared by the host planner (scan_plan.cpp) and the kernels.
#pragma once
#include <stdint.h>

#define CMGB_MAXC 6

// Per-state descriptor consumed by the kernels (one per state, indexed v).
struct StateInfo {
  int8_t  type;      // CMGB_*_st
  int8_t  kind;      // SK_* below
  int8_t  cnum;      // children (non-B); 0 for E
  int8_t  sd;        // StateDelta
  int8_t  right;     // reads children at row r-1 (MP, MR, IR)
  int8_t  emit;      // 0 none, 1 left, 2 right, 3 pair
  int8_t  has_begin; // local begin into this state
  int8_t  has_end;   // local end (init_sc not IMPOSSIBLE)
  int8_t  has_iend;  // integer version of has_end
  int8_t  pad_[3];
  int     v;         // state index
  int     next_off;  // byte offset of the next phase's record (desc + emission row) in the record array
  int     next_bytes;// its size (multiple of 16)
  // cell-walk constants for the kernel's thread count: padded range [lo,hi]
  // and band [dn,dxW]: width, step in rows / columns per nt cells
  int     wp_all, sr_all, sdd_all, wp_band, sr_band, sdd_band;
  float   inv_all, inv_band;    // 1/width, for the first row/column split
  int     next_carry, next_cw;  // carry row (offset, width) of the next phase in sweep order, -1: none;
                                // the kernel prefetches it one phase ahead
  int     lo, hi;    // padded d range of the buffer
  int     dn, dxW;   // own band for j >= W (dx shrinks to jp for small jp)
  int     buf;       // shared-memory element offset of row 0 (E: constant row)
  int     stride;    // elements per row (0 for E: every row is the d=0 init row)
  int     carry;     // element offset of [lo,hi] in the per-CTA carry arrays (-1: none)
  int     ring;      // BEGL_S: element offset of its history ring in the per-CTA ring area
  int     child[CMGB_MAXC];  // child state indices (non-B); B: child[0] = BEGL, child[1] = BEGR
  int     cbuf[CMGB_MAXC];   // child's buf, stride and lo (copied so a phase needs no pointer chase)
  int     cstr[CMGB_MAXC];
  int     clo[CMGB_MAXC];
  float   tsc[CMGB_MAXC];
  int     itsc[CMGB_MAXC];
  float   beginsc, endsc, init0;   // init0: value of the d = 0 cell
  int     ibeginsc, iendsc, iinit0;
  int     oesc_off;  // element offset of this state's emission row in the oesc/ioesc tables
  // B states: k range terms (src/cm_dpsearch.c:258-269)
  int     dn_y, dx_y, dn_w, dx_w, banded;
};

// Per-state descriptor of the truncated scan (RefTrCYKScan /
// RefITrInsideScan): the standard descriptor plus the truncated-begin
// penalties and the plane layout.  Every state keeps three score planes --
// J (joint), L (left marginal), R (right marginal) -- of (T+1) x stride cells
// each, mstride elements apart; its carry rows and, for BEGL_S, its history
// ring hold the same three planes.  The T (terminal) scores of bifurcations
// are only read by the root and go straight into its accumulators.
struct TrStateInfo {
  StateInfo s;          // s.buf / s.carry / s.ring address plane J
  float pty[3];         // truncated-begin penalty into this state, per penalty index (IMPOSSIBLE: none)
  int   ipty[3];        // integer penalties (-INFTY: none)
  int   mstride;        // elements between this state's planes (tile buffer)
  int   cm[CMGB_MAXC];  // children's plane strides (B: cm[0] is the BEGL ring's)
  int   iinit0;         // d = 0 value of the integer J plane
  int   pad_[2];
};

enum {
  SK_E = 0,      // end state: constant row, never computed
  SK_GEN = 1,    // generic: all cells independent
  SK_IL = 2,     // insert-left: self-loop on the current row (serial in d)
  SK_IR = 3,     // insert-right: self-loop on the previous row (serial along diagonals)
  SK_B = 4,      // bifurcation
  SK_BEGL = 5,   // BEGL_S: written to the global history ring
  SK_ROOT = 6,   // state 0
  SK_DET = 7     // truncated scans: detached insert (never computed, all IMPOSSIBLE)
};

// Whole-plan parameters (device copy lives in global memory).
struct ScanPlan {
  int M, W, T;            // states, model W, tile rows
  int nphase;             // computed states (all but E), processed in descending v
  int desc_off;           // element offset of the two prefetched phase descriptors
  int desc_words;         // words per descriptor (StateInfo)
  int rec_max_bytes;      // largest phase record (descriptor + emission row)
  int rec0_bytes;         // size of phase 0's record
  int esc_off;            // element offset of the two prefetched emission rows (Kp*Kp each)
  int tmp_off;            // element offset of the insert-state scratch [(T+1) x tmp_stride], in the
                          // tile arena or, when tmp_smem, in shared memory
  int tmp_stride;
  int acc_w;              // root accumulator width (root band)
  int ltbl_off;           // element offset of the uint16 ILogsum table (integer Inside plans only)
  int arena_global;       // 1: tile buffers, constant row, accumulator and insert scratch live in a
                          //    per-CTA global-memory arena (L1/L2 resident) instead of shared memory
  int arena_elems;        // size of that per-CTA arena (elements)
  int Kp;
  int nthreads;
  int smem_elems;         // tile-buffer arena size (elements of 4 bytes)
  int const_row;          // element offset of the shared constant E row
  int const_row_len;      // W + 2
  int acc_off;            // element offset of the root accumulator [T][W+1]
  int bestr_off;          // element offset of the bestr array [T][W+1] (ints)
  int res_off;            // element offset of the staged residues (bytes packed)
  int res_len;            // number of staged residues per tile (W + T + 2)
  int smem_bytes;         // total dynamic shared memory
  int carry_elems;        // per-CTA carry size (one parity)
  int ring_elems;         // per-CTA BEGL ring size
  int ring_rows;          // R
  int root_dn, root_dxW;
  float el_selfsc;
  int iel_selfsc;
  int local_begin;
  // truncated scans only
  int imp_row;            // element offset of an all-IMPOSSIBLE constant row (detached states)
  int rmax_off;           // element offset of the root's running maxima [4 modes][2 parities][acc_w]
  int tmp_smem;           // standard scans: the insert scratch lives in shared memory
};

#ifndef CMGB_NO_HOST_PLAN
#include <string>
#include <vector>
#include "../../include/infernal_gb300.h"
namespace cmgb {
struct PlanOut {
  ScanPlan plan;
  std::vector<StateInfo> states;   // indexed by state v
  std::vector<StateInfo> phases;   // computed states in sweep order (v = M-1 .. 0, E states left out)
  std::vector<unsigned char> records;  // per phase: StateInfo + its emission row, 16-byte aligned
  std::string err;
};
// Builds the plan of band set qdbidx with T-row tiles; false + err on failure.
bool build_plan(const cmgb_model_desc *m, int qdbidx, int T, int nthreads, bool logsum_table, bool arena_global, PlanOut *out);
// Packs the phase records (descriptor followed by the state's emission row,
// float or int) that the kernel streams into shared memory one phase ahead.
void build_records(const cmgb_model_desc *m, bool ins, PlanOut *out);

struct TrPlanOut {
  ScanPlan plan;
  std::vector<TrStateInfo> states;   // indexed by state v
  std::vector<TrStateInfo> phases;   // computed states in sweep order (E and detached states left out)
  std::string err;
};
// Plan of the truncated scan of band set qdbidx: every state's band is
// d = 1 .. min(dmax, W) (src/cm_mx.c:6432-6438).  Requires the model's
// truncation tables (lmesc/rmesc, penalties); false + err otherwise.
bool build_tr_plan(const cmgb_model_desc *m, int qdbidx, int T, int nthreads, bool logsum_table, bool arena_global, TrPlanOut *out);
}  // namespace cmgb
#endif
