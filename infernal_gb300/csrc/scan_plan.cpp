// scan_plan.cpp -- builds the per-(model, band set, tile size) ScanPlan.
//
// Band arithmetic follows cm_scan_mx_Create (src/cm_mx.c:5725-5738):
//   dn(v) = min(max(dmin(v), MP ? 2 : 1), W),  dx(v, jp) = min(jp, dmax(v), W)
// and the B-state k limits of FastCYKScan (src/cm_dpsearch.c:258-269).
// The d = 0 cell values follow cm_scan_mx_InitializeFloats/Integers
// (src/cm_mx.c:6039-6138).
#include "scan_plan.h"
#include "../../include/infernal_gb300.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

static_assert(sizeof(StateInfo) % 16 == 0, "phase records must stay 16-byte aligned");

namespace cmgb {

static inline int st_delta(int t) { return t == CMGB_MP_st ? 2 : (t == CMGB_ML_st || t == CMGB_MR_st || t == CMGB_IL_st || t == CMGB_IR_st) ? 1 : 0; }
static inline bool st_right(int t) { return t == CMGB_MP_st || t == CMGB_MR_st || t == CMGB_IR_st; }

// First-fit arena allocator over [0, inf) in elements.
struct Arena {
  std::vector<std::pair<int, int>> used;  // (offset, size), sorted by offset
  int peak = 0;
  int alloc(int size) {
    int off = 0;
    for (size_t k = 0; k < used.size(); k++) {
      if (used[k].first - off >= size) { used.insert(used.begin() + k, {off, size}); peak = std::max(peak, off + size); return off; }
      off = used[k].first + used[k].second;
    }
    used.push_back({off, size});
    peak = std::max(peak, off + size);
    return off;
  }
  void release(int off) {
    for (size_t k = 0; k < used.size(); k++) if (used[k].first == off) { used.erase(used.begin() + k); return; }
  }
};

bool build_plan(const cmgb_model_desc *m, int qdbidx, int T, int nthreads, bool logsum_table, bool arena_global, PlanOut *out)
{
  const int M = m->M, Wm = m->W;
  const int *dmin = qdbidx == CMGB_QDB1_TIGHT ? m->dmin1 : qdbidx == CMGB_QDB2_LOOSE ? m->dmin2 : nullptr;
  const int *dmax = qdbidx == CMGB_QDB1_TIGHT ? m->dmax1 : qdbidx == CMGB_QDB2_LOOSE ? m->dmax2 : nullptr;
  std::vector<StateInfo> S(M);
  std::memset(S.data(), 0, sizeof(StateInfo) * M);

  // -- bands and static per-state fields
  for (int v = 0; v < M; v++) {
    StateInfo &s = S[v];
    int t = m->sttype[v];
    s.type = (int8_t) t;
    s.sd = (int8_t) st_delta(t);
    s.right = (int8_t) st_right(t);
    s.emit = (t == CMGB_MP_st) ? 3 : (t == CMGB_ML_st || t == CMGB_IL_st) ? 1 : (t == CMGB_MR_st || t == CMGB_IR_st) ? 2 : 0;
    int lo = t == CMGB_MP_st ? 2 : 1;
    if (dmin) lo = std::max(dmin[v], lo);
    s.dn = std::min(lo, Wm);
    s.dxW = dmax ? std::min(dmax[v], Wm) : Wm;
    if (v == 0) s.kind = SK_ROOT;
    else if (t == CMGB_E_st) s.kind = SK_E;
    else if (t == CMGB_B_st) s.kind = SK_B;
    else if (m->stid[v] == CMGB_BEGL_S) s.kind = SK_BEGL;
    else if (t == CMGB_IL_st) s.kind = SK_IL;
    else if (t == CMGB_IR_st) s.kind = SK_IR;
    else s.kind = SK_GEN;
    if (t == CMGB_B_st) {
      s.cnum = 2;
      s.child[0] = m->cfirst[v];  // BEGL_S
      s.child[1] = m->cnum[v];    // BEGR_S
      int w = s.child[0], y = s.child[1];
      s.banded = dmin != nullptr;
      if (dmin) {
        s.dn_y = std::min(dmin[y], Wm); s.dx_y = std::min(dmax[y], Wm);
        s.dn_w = std::min(dmin[w], Wm); s.dx_w = std::min(dmax[w], Wm);
      }
    } else if (t != CMGB_E_st) {
      s.cnum = (int8_t) m->cnum[v];
      if (s.kind != SK_ROOT && s.kind != SK_BEGL && (m->cnum[v] < 2 || m->cnum[v] > 6)) {
        out->err = "state " + std::to_string(v) + " has an unsupported child count " + std::to_string(m->cnum[v]);
        return false;
      }
      if (m->cnum[v] > CMGB_MAXC || m->cnum[v] < 1) { out->err = "bad child count"; return false; }
      for (int o = 0; o < m->cnum[v]; o++) {
        s.child[o] = m->cfirst[v] + o;
        s.tsc[o] = m->tsc[v * 6 + o];
        s.itsc[o] = m->itsc[v * 6 + o];
      }
    }
    s.beginsc = m->beginsc[v]; s.ibeginsc = m->ibeginsc[v];
    s.endsc = m->endsc[v]; s.iendsc = m->iendsc[v];
    s.has_begin = (m->flags & CMGB_LOCAL_BEGIN) && v > 0 && (m->beginsc[v] > -9.999e35f);
    s.has_end = m->endsc[v] > -9.999e35f;
    s.has_iend = m->iendsc[v] != -CMGB_INFTY;
    s.oesc_off = v * m->Kp * m->Kp;
    s.carry = -1; s.ring = -1; s.buf = -1;
    s.v = v;
  }
  // Integer local-begin availability must agree with the float one
  for (int v = 1; v < M; v++)
    if (((m->flags & CMGB_LOCAL_BEGIN) && m->ibeginsc[v] != -CMGB_INFTY) != (bool) S[v].has_begin) {
      out->err = "beginsc/ibeginsc disagree on local begin states"; return false;
    }

  // -- d = 0 values (src/cm_mx.c:6039-6138), children before parents
  std::vector<float> f0(M, CMGB_IMPOSSIBLE);
  std::vector<int> i0(M, -CMGB_INFTY);
  for (int v = M - 1; v >= 0; v--) {
    int t = m->sttype[v];
    if (m->stid[v] == CMGB_BEGL_S || t == CMGB_S_st || t == CMGB_D_st) {
      float fs = m->endsc[v]; int is = m->iendsc[v];
      for (int o = 0; o < m->cnum[v]; o++) {
        float c = f0[m->cfirst[v] + o] + m->tsc[v * 6 + o]; fs = fs > c ? fs : c;
        int ic = i0[m->cfirst[v] + o] + m->itsc[v * 6 + o]; is = is > ic ? is : ic;
      }
      f0[v] = fs > CMGB_IMPOSSIBLE ? fs : CMGB_IMPOSSIBLE;
      i0[v] = is > -CMGB_INFTY ? is : -CMGB_INFTY;
    } else if (t == CMGB_E_st) { f0[v] = 0.f; i0[v] = 0; }
    else if (t == CMGB_B_st) {
      f0[v] = f0[m->cfirst[v]] + f0[m->cnum[v]];
      i0[v] = i0[m->cfirst[v]] + i0[m->cnum[v]];
    }
    S[v].init0 = f0[v]; S[v].iinit0 = i0[v];
  }

  // -- padded buffer ranges: own band plus every parent read
  for (int v = 0; v < M; v++) { S[v].lo = S[v].dn; S[v].hi = S[v].dxW; }
  auto widen = [&](int y, int lo, int hi) { if (lo <= hi) { S[y].lo = std::min(S[y].lo, lo); S[y].hi = std::max(S[y].hi, hi); } };
  std::vector<int> last_use(M, -1);   // smallest parent index (processed last)
  for (int p = 0; p < M; p++) {
    const StateInfo &s = S[p];
    if (s.kind == SK_E) continue;
    if (s.kind == SK_B) {
      int w = s.child[0], y = s.child[1];
      for (int d = s.dn; d <= s.dxW; d++) {
        int kmin = s.banded ? std::max(0, std::max(s.dn_y, d - s.dx_w)) : 0;
        int kmax = s.banded ? std::min(s.dx_y, d - s.dn_w) : d;
        if (kmin > kmax) continue;
        widen(y, kmin, kmax);
        widen(w, d - kmax, d - kmin);
      }
      if (last_use[y] < 0 || p < last_use[y]) last_use[y] = p;
      continue;
    }
    int rlo = s.dn - s.sd, rhi = s.dxW - s.sd;
    for (int o = 0; o < s.cnum; o++) {
      int y = s.child[o];
      widen(y, rlo, rhi);
      if (y != p && (last_use[y] < 0 || p < last_use[y])) last_use[y] = p;
    }
  }
  for (int v = 0; v < M; v++) { if (S[v].lo < 0) S[v].lo = 0; if (S[v].hi > Wm) S[v].hi = Wm; if (S[v].hi < S[v].lo) S[v].hi = S[v].lo; }

  // -- shared-memory arena for tile buffers (interval allocation in sweep order)
  Arena arena;
  std::vector<std::vector<int>> free_after(M + 1);   // free_after[u]: buffers whose last reader is state u
  int carry = 0, ring = 0;
  const int R = Wm + T + 1;
  for (int v = M - 1; v >= 0; v--) {
    StateInfo &s = S[v];
    if (v + 1 < M) { for (int y : free_after[v + 1]) arena.release(S[y].buf); free_after[v + 1].clear(); }
    if (s.kind == SK_E) { s.stride = 0; s.lo = 0; continue; }
    int width = s.hi - s.lo + 1;
    if (s.kind == SK_BEGL) {         // history ring in global memory, no tile buffer
      s.stride = width;
      s.ring = ring; ring += R * width;
      continue;
    }
    if (s.kind == SK_ROOT) { s.stride = width; continue; }   // folded straight into the accumulator
    s.stride = width | 1;   // odd stride: one column of the T rows spans distinct banks
    s.buf = arena.alloc((T + 1) * s.stride);
    s.carry = carry; carry += s.stride;
    int lu = last_use[v] < 0 ? v : last_use[v];
    free_after[lu].push_back(v);
  }

  ScanPlan P;
  std::memset(&P, 0, sizeof(P));
  P.M = M; P.W = Wm; P.T = T; P.Kp = m->Kp; P.nthreads = nthreads;
  int tmp_stride = 1;
  for (int v = 0; v < M; v++) if (S[v].kind == SK_IL || S[v].kind == SK_IR) tmp_stride = std::max(tmp_stride, S[v].hi - S[v].lo + 1);
  tmp_stride |= 1;
  int off = arena.peak;
  off = (off + 3) & ~3;
  P.const_row = off; P.const_row_len = Wm + 2; off += (Wm + 2 + 3) & ~3;
  P.acc_w = std::max(1, S[0].dxW - S[0].dn + 1);
  P.acc_off = off; off += T * P.acc_w;
  P.bestr_off = off; off += T * P.acc_w;
  P.tmp_stride = tmp_stride;
  const int tmp_elems = (T + 1) * tmp_stride;
  // the insert scratch is read back by the self-loop chains right after it is
  // written; with a global arena it still goes to shared memory when it fits
  // next to the ILogsum table, the residues and the phase records
  P.tmp_smem = !arena_global || tmp_elems * 4 + (logsum_table ? CMGB_LOGSUM_TBL * 2 : 0) + 4 * (Wm + T) <= 176 * 1024;
  if (!P.tmp_smem) { P.tmp_off = off; off += tmp_elems; }
  off = (off + 3) & ~3;
  P.arena_global = arena_global ? 1 : 0;
  if (arena_global) {            // everything above goes to global memory; shared memory restarts at 0
    P.arena_elems = off;
    off = 0;
  } else P.arena_elems = 0;
  if (P.tmp_smem) { P.tmp_off = off; off += tmp_elems; off = (off + 3) & ~3; }
  P.desc_words = (int) (sizeof(StateInfo) / 4);
  P.rec_max_bytes = (int) sizeof(StateInfo) + ((m->Kp * m->Kp * 4 + 15) & ~15);
  P.desc_off = off; off += 2 * (P.rec_max_bytes / 4);     // two record slots, 16-byte aligned
  P.esc_off = P.desc_off + P.desc_words;                  // emission row follows the descriptor in a slot
  off = (off + 3) & ~3;
  P.res_off = off; P.res_len = Wm + T + 2; off += (P.res_len + 3) / 4;
  off = (off + 3) & ~3;
  P.ltbl_off = off;
  if (logsum_table) off += (CMGB_LOGSUM_TBL * 2 + 3) / 4;
  P.smem_elems = off;
  P.smem_bytes = off * 4 + 32;   // + the window slot and the two record mbarriers
  P.carry_elems = carry;
  P.ring_elems = ring > 0 ? ring : 1;
  P.ring_rows = R;
  P.root_dn = S[0].dn; P.root_dxW = S[0].dxW;
  P.el_selfsc = m->el_selfsc; P.iel_selfsc = m->iel_selfsc;
  P.local_begin = (m->flags & CMGB_LOCAL_BEGIN) ? 1 : 0;
  for (int v = 0; v < M; v++) if (S[v].kind == SK_E) S[v].buf = P.const_row;
  for (int v = 0; v < M; v++) {
    StateInfo &s = S[v];
    if (s.kind == SK_E) continue;
    for (int o = 0; o < s.cnum && o < CMGB_MAXC; o++) {
      const StateInfo &c = S[s.child[o]];
      s.cbuf[o] = c.kind == SK_BEGL ? c.ring : c.buf;
      s.cstr[o] = c.stride;
      s.clo[o] = c.lo;
    }
  }
  P.nphase = 0;
  for (int v = 0; v < M; v++) {
    StateInfo &q = S[v];
    q.wp_all = std::max(1, q.hi - q.lo + 1); q.sr_all = nthreads / q.wp_all; q.sdd_all = nthreads - q.sr_all * q.wp_all;
    q.wp_band = std::max(1, q.dxW - q.dn + 1); q.sr_band = nthreads / q.wp_band; q.sdd_band = nthreads - q.sr_band * q.wp_band;
    q.inv_all = 1.0f / (float) q.wp_all; q.inv_band = 1.0f / (float) q.wp_band;
  }
  for (int v = M - 1; v >= 0; v--) if (S[v].kind != SK_E) { out->phases.push_back(S[v]); P.nphase++; }
  for (size_t k = 0; k < out->phases.size(); k++) {
    const bool nx = k + 1 < out->phases.size() && out->phases[k + 1].carry >= 0;
    out->phases[k].next_carry = nx ? out->phases[k + 1].carry : -1;
    out->phases[k].next_cw = nx ? out->phases[k + 1].hi - out->phases[k + 1].lo + 1 : 0;
  }
  out->plan = P;
  out->states = std::move(S);
  return true;
}

}  // namespace cmgb

namespace cmgb {
void build_records(const cmgb_model_desc *m, bool ins, PlanOut *out)
{
  const int KK = m->Kp * m->Kp;
  std::vector<int> off(out->phases.size()), bytes(out->phases.size());
  size_t total = 0;
  for (size_t k = 0; k < out->phases.size(); k++) {
    const StateInfo &s = out->phases[k];
    int elen = s.emit == 3 ? KK : s.emit ? m->Kp : 0;
    bytes[k] = (int) sizeof(StateInfo) + ((elen * 4 + 15) & ~15);
    off[k] = (int) total;
    total += bytes[k];
  }
  out->records.assign(total, 0);
  const size_t np = out->phases.size();
  for (size_t k = 0; k < np; k++) {
    StateInfo s = out->phases[k];
    s.next_off = off[(k + 1) % np];
    s.next_bytes = bytes[(k + 1) % np];
    out->phases[k].next_off = s.next_off;
    out->phases[k].next_bytes = s.next_bytes;
    std::memcpy(&out->records[off[k]], &s, sizeof(StateInfo));
    int elen = s.emit == 3 ? KK : s.emit ? m->Kp : 0;
    unsigned char *e = &out->records[off[k] + sizeof(StateInfo)];
    for (int q = 0; q < elen; q++) {
      if (ins) { int x = m->ioesc[(size_t) s.v * KK + q]; std::memcpy(e + 4 * q, &x, 4); }
      else { float x = m->oesc[(size_t) s.v * KK + q]; std::memcpy(e + 4 * q, &x, 4); }
    }
  }
  out->plan.rec0_bytes = bytes[0];
}
}  // namespace cmgb

// ---------------------------------------------------------------------------
// Truncated scan plan (RefTrCYKScan / RefITrInsideScan,
// src/cm_dpsearch_trunc.c:79-1338).  Bands: d = 1 .. min(dmax, W) for every
// state (src/cm_mx.c:6432-6438).  d = 0 cells of the J plane follow
// cm_tr_scan_mx_InitializeFloats/Integers (src/cm_mx.c:6853-6960); the integer
// version starts its S/D/BEGL cells from the float endsc converted to int,
// as the reference does.  L/R planes hold IMPOSSIBLE at d = 0 except for E.
namespace cmgb {

// C's float -> int conversion (truncation; IMPOSSIBLE saturates to INT_MIN)
static inline int c_f2i(float x) { return x > -2147483648.0f ? (int) x : (int) 0x80000000; }

bool build_tr_plan(const cmgb_model_desc *m, int qdbidx, int T, int nthreads, bool logsum_table, bool arena_global, TrPlanOut *out)
{
  const int M = m->M, Wm = m->W;
  if (!m->lmesc || !m->rmesc || !m->ilmesc || !m->irmesc || !m->tr_g_pty || !m->tr_l_pty || !m->tr_ig_pty || !m->tr_il_pty) {
    out->err = "model has no truncation tables (lmesc/rmesc and truncated-begin penalties)";
    return false;
  }
  const int *dmax = qdbidx == CMGB_QDB1_TIGHT ? m->dmax1 : qdbidx == CMGB_QDB2_LOOSE ? m->dmax2 : nullptr;
  const bool local = (m->flags & CMGB_LOCAL_BEGIN) != 0;
  std::vector<TrStateInfo> S(M);
  std::memset(S.data(), 0, sizeof(TrStateInfo) * M);
  for (int v = 0; v < M; v++) {
    TrStateInfo &ti = S[v];
    StateInfo &s = ti.s;
    const int t = m->sttype[v];
    s.type = (int8_t) t;
    s.sd = (int8_t) st_delta(t);
    s.right = (int8_t) st_right(t);
    s.emit = (t == CMGB_MP_st) ? 3 : (t == CMGB_ML_st || t == CMGB_IL_st) ? 1 : (t == CMGB_MR_st || t == CMGB_IR_st) ? 2 : 0;
    s.dn = 1;
    s.dxW = dmax ? std::min(dmax[v], Wm) : Wm;
    const bool detached = v + 1 < M && m->stid[v + 1] == CMGB_END_E && (t == CMGB_IL_st || t == CMGB_IR_st || t == CMGB_ML_st || t == CMGB_MR_st);
    if (v == 0) s.kind = SK_ROOT;
    else if (t == CMGB_E_st) s.kind = SK_E;
    else if (detached) s.kind = SK_DET;
    else if (t == CMGB_B_st) s.kind = SK_B;
    else if (m->stid[v] == CMGB_BEGL_S) s.kind = SK_BEGL;
    else if (t == CMGB_IL_st) s.kind = SK_IL;
    else if (t == CMGB_IR_st) s.kind = SK_IR;
    else s.kind = SK_GEN;
    if (t == CMGB_B_st) {
      s.cnum = 2;
      s.child[0] = m->cfirst[v];   // BEGL_S
      s.child[1] = m->cnum[v];     // BEGR_S
      s.banded = dmax != nullptr;
      if (dmax) { s.dx_y = std::min(dmax[s.child[1]], Wm); s.dx_w = std::min(dmax[s.child[0]], Wm); }
    } else if (t != CMGB_E_st && v > 0) {
      if (m->cnum[v] < 1 || m->cnum[v] > CMGB_MAXC) { out->err = "state " + std::to_string(v) + " has an unsupported child count"; return false; }
      s.cnum = (int8_t) m->cnum[v];
      for (int o = 0; o < m->cnum[v]; o++) {
        s.child[o] = m->cfirst[v] + o;
        s.tsc[o] = m->tsc[v * 6 + o];
        s.itsc[o] = m->itsc[v * 6 + o];
      }
    }
    s.endsc = m->endsc[v]; s.iendsc = m->iendsc[v];
    s.has_end = m->endsc[v] > -9.999e35f;
    s.has_iend = m->iendsc[v] != -CMGB_INFTY;
    s.oesc_off = v * m->Kp * m->Kp;
    s.carry = -1; s.ring = -1; s.buf = -1;
    s.v = v;
    for (int p = 0; p < 3; p++) {
      ti.pty[p] = (local ? m->tr_l_pty : m->tr_g_pty)[(size_t) p * M + v];
      ti.ipty[p] = (local ? m->tr_il_pty : m->tr_ig_pty)[(size_t) p * M + v];
    }
    // truncated begins never enter BEGL_S (src/cm_dpsearch_trunc.c:545); E
    // and detached states only ever hold IMPOSSIBLE scores
    if (s.kind == SK_BEGL || s.kind == SK_E || s.kind == SK_ROOT) {
      for (int p = 0; p < 3; p++) { ti.pty[p] = CMGB_IMPOSSIBLE; ti.ipty[p] = -CMGB_INFTY; }
    }
  }
  // d = 0 cells of the J planes, children before parents
  std::vector<float> f0(M, CMGB_IMPOSSIBLE);
  std::vector<int> i0(M, -CMGB_INFTY);
  for (int v = M - 1; v >= 0; v--) {
    const int t = m->sttype[v];
    if (m->stid[v] == CMGB_BEGL_S || t == CMGB_S_st || t == CMGB_D_st) {
      float fs = m->endsc[v]; int is = c_f2i(m->endsc[v]);
      for (int o = 0; o < m->cnum[v]; o++) {
        float c = f0[m->cfirst[v] + o] + m->tsc[v * 6 + o]; fs = fs > c ? fs : c;
        int ic = i0[m->cfirst[v] + o] + m->itsc[v * 6 + o]; is = is > ic ? is : ic;
      }
      f0[v] = fs > CMGB_IMPOSSIBLE ? fs : CMGB_IMPOSSIBLE;
      i0[v] = is > -CMGB_INFTY ? is : -CMGB_INFTY;
    } else if (t == CMGB_E_st) { f0[v] = 0.f; i0[v] = 0; }
    else if (t == CMGB_B_st) {
      f0[v] = f0[m->cfirst[v]] + f0[m->cnum[v]];
      i0[v] = i0[m->cfirst[v]] + i0[m->cnum[v]];
    }
    S[v].s.init0 = f0[v]; S[v].iinit0 = i0[v];
  }
  // padded ranges: [0, max(own band, every parent's band)]; last reader of each buffer
  for (int v = 0; v < M; v++) { S[v].s.lo = 0; S[v].s.hi = S[v].s.dxW; }
  std::vector<int> last_use(M, -1);
  for (int p = 0; p < M; p++) {
    const StateInfo &s = S[p].s;
    if (s.kind == SK_E || s.kind == SK_DET || s.kind == SK_ROOT) continue;   // the root reads no child buffer here
    for (int o = 0; o < s.cnum; o++) {
      const int y = s.child[o];
      S[y].s.hi = std::max(S[y].s.hi, s.dxW);
      if (y != p && (last_use[y] < 0 || p < last_use[y])) last_use[y] = p;
    }
  }
  for (int v = 0; v < M; v++) if (S[v].s.hi > Wm) S[v].s.hi = Wm;

  // arena: three planes of (T+1) rows per live state, interval allocation in sweep order
  Arena arena;
  std::vector<std::vector<int>> free_after(M + 1);
  int carry = 0, ring = 0;
  const int RR = Wm + T + 1;
  for (int v = M - 1; v >= 0; v--) {
    TrStateInfo &ti = S[v];
    StateInfo &s = ti.s;
    if (v + 1 < M) { for (int y : free_after[v + 1]) arena.release(S[y].s.buf); free_after[v + 1].clear(); }
    if (s.kind == SK_E || s.kind == SK_DET) { s.stride = 0; ti.mstride = 0; continue; }
    const int width = s.hi - s.lo + 1;
    if (s.kind == SK_BEGL) {
      s.stride = width;
      ti.mstride = RR * width;
      s.ring = ring; ring += 3 * RR * width;
      continue;
    }
    if (s.kind == SK_ROOT) { s.stride = width; continue; }
    s.stride = width | 1;
    ti.mstride = (T + 1) * s.stride;
    s.buf = arena.alloc(3 * ti.mstride);
    s.carry = carry; carry += 3 * s.stride;
    const int lu = last_use[v] < 0 ? v : last_use[v];
    free_after[lu].push_back(v);
  }

  ScanPlan P;
  std::memset(&P, 0, sizeof(P));
  P.M = M; P.W = Wm; P.T = T; P.Kp = m->Kp; P.nthreads = nthreads;
  int off = (arena.peak + 3) & ~3;
  P.const_row = off; P.const_row_len = Wm + 2; off += (Wm + 2 + 3) & ~3;
  P.imp_row = off; off += (Wm + 2 + 3) & ~3;
  P.acc_w = std::max(1, S[0].s.dxW);
  P.acc_off = off; off += 4 * T * P.acc_w;
  P.bestr_off = off; off += 4 * T * P.acc_w;
  P.rmax_off = off; off += 8 * P.acc_w;
  off = (off + 3) & ~3;
  P.arena_global = arena_global ? 1 : 0;
  if (arena_global) { P.arena_elems = off; off = 0; } else P.arena_elems = 0;
  P.res_off = off; P.res_len = Wm + T + 2; off += (P.res_len + 3) / 4;
  off = (off + 3) & ~3;
  P.ltbl_off = off;
  if (logsum_table) off += (CMGB_LOGSUM_TBL * 2 + 3) / 4;
  // CYK only: the inserts' non-self terms of the two self-loop planes (IL:
  // J and L, IR: J and R), read back by the self-loop chains; in shared
  // memory (the order-free max lets the chains fold them last)
  if (!logsum_table) {
    int tstr = 1;
    for (int v = 0; v < M; v++) if (S[v].s.kind == SK_IL || S[v].s.kind == SK_IR) tstr = std::max(tstr, S[v].s.hi - S[v].s.lo + 1);
    P.tmp_stride = tstr | 1;
    off = (off + 3) & ~3;
    P.tmp_off = off; P.tmp_smem = 1;
    off += 2 * (T + 1) * P.tmp_stride;
  }
  P.smem_elems = off;
  P.smem_bytes = off * 4 + 32;
  P.carry_elems = carry;
  P.ring_elems = ring > 0 ? ring : 1;
  P.ring_rows = RR;
  P.root_dn = 1; P.root_dxW = S[0].s.dxW;
  P.el_selfsc = m->el_selfsc; P.iel_selfsc = m->iel_selfsc;
  P.local_begin = (m->flags & CMGB_LOCAL_BEGIN) ? 1 : 0;
  for (int v = 0; v < M; v++) {
    if (S[v].s.kind == SK_E) S[v].s.buf = P.const_row;
    if (S[v].s.kind == SK_DET) S[v].s.buf = P.imp_row;
  }
  for (int v = 0; v < M; v++) {
    TrStateInfo &ti = S[v];
    StateInfo &s = ti.s;
    if (s.kind == SK_E || s.kind == SK_DET) continue;
    for (int o = 0; o < s.cnum && o < CMGB_MAXC; o++) {
      const TrStateInfo &c = S[s.child[o]];
      s.cbuf[o] = c.s.kind == SK_BEGL ? c.s.ring : c.s.buf;
      s.cstr[o] = c.s.stride;
      s.clo[o] = c.s.lo;
      ti.cm[o] = c.mstride;
    }
  }
  P.nphase = 0;
  for (int v = 0; v < M; v++) {
    StateInfo &q = S[v].s;
    q.wp_all = std::max(1, q.hi - q.lo + 1); q.sr_all = nthreads / q.wp_all; q.sdd_all = nthreads - q.sr_all * q.wp_all;
    q.wp_band = std::max(1, q.dxW - q.dn + 1); q.sr_band = nthreads / q.wp_band; q.sdd_band = nthreads - q.sr_band * q.wp_band;
    q.inv_all = 1.0f / (float) q.wp_all; q.inv_band = 1.0f / (float) q.wp_band;
  }
  for (int v = M - 1; v >= 0; v--)
    if (S[v].s.kind != SK_E && S[v].s.kind != SK_DET) { out->phases.push_back(S[v]); P.nphase++; }
  for (auto &ph : out->phases) { ph.s.next_carry = -1; ph.s.next_cw = 0; }
  out->plan = P;
  out->states = std::move(S);
  return true;
}

}  // namespace cmgb
