/* cm_tr_oracle_core.h -- typed DP core of the truncated scanners, included by
 * cm_scan_oracle.c once per score semiring.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates RefTrCYKScan (src/cm_dpsearch_trunc.c:79-700; semiring max) and
 * RefITrInsideScan (src/cm_dpsearch_trunc.c:741-1338; semiring ILogsum): the
 * J (joint), L (left-marginal), R (right-marginal) matrices for every state
 * and T for bifurcations, one end position j at a time, states v = M-1..1,
 * then the root's truncated begins.  Combination order inside each cell is
 * the reference's: the init score first, then the children in yoffset order.
 *
 * Expected macros: TR_CORE_NAME, SCT, IMPV, COMB(a,b), IS_PTY(p), SCOREF(x),
 * TSC(v,o), ESC(v), LMESC(v), RMESC(v), PTY(y), INIT_SC(v,d), RUNNING_VSC.
 */
static void TR_CORE_NAME(scanctx *c)
{
  const cmgb_model_desc *m = c->m;
  const int M = c->M, W = c->W, WP = W + 1, Kp = c->Kp;
  const int fill_L = c->fill_L, fill_R = c->fill_R, fill_T = c->fill_T;
  const uint8_t *dsq = c->dsq;
  const size_t plane = (size_t) M * WP;
  SCT *Jm = malloc(sizeof(SCT) * 2 * plane), *Lm = malloc(sizeof(SCT) * 2 * plane);
  SCT *Rm = malloc(sizeof(SCT) * 2 * plane), *Tm = malloc(sizeof(SCT) * 2 * plane);
  const size_t bplane = (size_t) WP * WP;     /* one BEGL deck: [row j%(W+1)][d] */
  SCT *Jb = malloc(sizeof(SCT) * (c->nbegl ? c->nbegl : 1) * bplane);
  SCT *Lb = malloc(sizeof(SCT) * (c->nbegl ? c->nbegl : 1) * bplane);
  SCT *Rb = malloc(sizeof(SCT) * (c->nbegl ? c->nbegl : 1) * bplane);
#define XJ(p, v, d) Jm[((size_t) (p) * M + (v)) * WP + (d)]
#define XL(p, v, d) Lm[((size_t) (p) * M + (v)) * WP + (d)]
#define XR(p, v, d) Rm[((size_t) (p) * M + (v)) * WP + (d)]
#define XT(p, v, d) Tm[((size_t) (p) * M + (v)) * WP + (d)]
#define BJ(r, v, d) Jb[(size_t) c->beglidx[v] * bplane + (size_t) (r) * WP + (d)]
#define BL(r, v, d) Lb[(size_t) c->beglidx[v] * bplane + (size_t) (r) * WP + (d)]
#define BR(r, v, d) Rb[(size_t) c->beglidx[v] * bplane + (size_t) (r) * WP + (d)]
  for (size_t q = 0; q < 2 * plane; q++) Jm[q] = Lm[q] = Rm[q] = Tm[q] = IMPV;
  for (size_t q = 0; q < (size_t) (c->nbegl ? c->nbegl : 1) * bplane; q++) Jb[q] = Lb[q] = Rb[q] = IMPV;

  /* d = 0 cells (cm_tr_scan_mx_InitializeFloats/Integers, src/cm_mx.c:6853-6960) */
  for (int v = M - 1; v >= 0; v--) {
    const int t = m->sttype[v];
    if (m->stid[v] != CMGB_BEGL_S) {
      if (t == CMGB_E_st) {
        XJ(0, v, 0) = XJ(1, v, 0) = 0; XL(0, v, 0) = XL(1, v, 0) = 0; XR(0, v, 0) = XR(1, v, 0) = 0;
        continue;
      } else if (t == CMGB_S_st || t == CMGB_D_st) {
        SCT s0 = ENDSC(v);
        for (int o = 0; o < m->cnum[v]; o++) s0 = MAXF(s0, XJ(0, m->cfirst[v] + o, 0) + TSC(v, o));
        XJ(0, v, 0) = MAXF(s0, IMPV);
      } else if (t == CMGB_B_st) {
        XJ(0, v, 0) = BJ(0, m->cfirst[v], 0) + XJ(0, m->cnum[v], 0);
      }
      XJ(1, v, 0) = XJ(0, v, 0);
    } else {
      SCT s0 = ENDSC(v);
      for (int o = 0; o < m->cnum[v]; o++) s0 = MAXF(s0, XJ(0, m->cfirst[v] + o, 0) + TSC(v, o));
      s0 = MAXF(s0, IMPV);
      for (int r = 0; r <= W; r++) BJ(r, v, 0) = s0;
    }
  }

  int *dxA = malloc(sizeof(int) * M);
  for (int64_t j = c->i0; j <= c->j0; j++) {
    const int64_t jp_g = j - c->i0 + 1;
    const int cur = (int) (j % 2), prv = (int) ((j - 1) % 2);
    const int jrow = jp_g >= W ? W : (int) jp_g;   /* dx uses row min(jp, W) */
    for (int v = 0; v < M; v++) dxA[v] = MINF(jrow, c->dxW[v]);
    if (c->act) {   /* residue counts for NULL3 (src/cm_dpsearch_trunc.c:882-886) */
      memcpy(c->act[jp_g % WP], c->act[(jp_g - 1) % WP], sizeof(double) * 8);
      count_residue(c->act[jp_g % WP], dsq[j], c->K);
    }
    for (int v = M - 1; v > 0; v--) {
      const int t = m->sttype[v];
      if (t == CMGB_E_st) continue;
      const int y = m->cfirst[v], cn = m->cnum[v];
      const int detached = (v + 1 < M) && m->stid[v + 1] == CMGB_END_E;
      if (t == CMGB_B_st) {
        const int w = m->cfirst[v], z = m->cnum[v];
        for (int d = 1; d <= dxA[v]; d++) {
          int kmin = 0, kmax = d;
          if (c->dmax) { kmin = MAXF(0, d - MINF(c->dmax[w], c->Wm)); kmax = MINF(MINF(c->dmax[z], c->Wm), d); }
          SCT Js = INIT_SC(v, d), Ls = INIT_SC(v, d), Rs = INIT_SC(v, d), Ts = INIT_SC(v, d);
          for (int k = kmin; k <= kmax; k++) {
            const int r = (int) ((j - k) % WP);
            Js = COMB(Js, BJ(r, w, d - k) + XJ(cur, z, k));
            if (fill_L) Ls = COMB(Ls, BJ(r, w, d - k) + XL(cur, z, k));
            if (fill_R) Rs = COMB(Rs, BR(r, w, d - k) + XJ(cur, z, k));
          }
          if (fill_T)
            for (int k = MAXF(1, kmin); k <= MINF(d - 1, kmax); k++) {
              const int r = (int) ((j - k) % WP);
              Ts = COMB(Ts, BR(r, w, d - k) + XL(cur, z, k));
            }
          XJ(cur, v, d) = Js;
          if (fill_T) XT(cur, v, d) = Ts;
          if (fill_L) {
            const int r0 = (int) (j % WP);
            XL(cur, v, d) = kmin == 0 ? COMB(Ls, MAXF(BJ(r0, w, d), BL(r0, w, d))) : Ls;
          }
          if (fill_R) XR(cur, v, d) = kmax == d ? COMB(Rs, MAXF(XJ(cur, z, d), XR(cur, z, d))) : Rs;
        }
      } else if (m->stid[v] == CMGB_BEGL_S) {
        const int r0 = (int) (j % WP);
        for (int d = 1; d <= dxA[v]; d++) {
          SCT Js = INIT_SC(v, d), Ls = INIT_SC(v, d), Rs = INIT_SC(v, d);
          for (int o = 0; o < cn; o++) {
            Js = COMB(Js, XJ(cur, y + o, d) + TSC(v, o));
            if (fill_L) Ls = COMB(Ls, XL(cur, y + o, d) + TSC(v, o));
            if (fill_R) Rs = COMB(Rs, XR(cur, y + o, d) + TSC(v, o));
          }
          BJ(r0, v, d) = Js;
          if (fill_L) BL(r0, v, d) = Ls;
          if (fill_R) BR(r0, v, d) = Rs;
        }
      } else if (t == CMGB_ML_st || t == CMGB_IL_st) {
        if (!detached) {
          const int R0 = t == CMGB_IL_st ? 1 : 0;
          for (int d = 1; d <= dxA[v]; d++) {
            const SCT e = ESC(v)[dsq[j - d + 1]];
            SCT Js = INIT_SC(v, d - 1), Ls = INIT_SC(v, d - 1), Rs = INIT_SC(v, d);
            if (fill_R) XR(cur, v, d) = Rs;
            for (int o = 0; o < cn; o++) {
              Js = COMB(Js, XJ(cur, y + o, d - 1) + TSC(v, o));
              if (fill_L) Ls = COMB(Ls, XL(cur, y + o, d - 1) + TSC(v, o));
            }
            XJ(cur, v, d) = Js + e;
            if (fill_L) XL(cur, v, d) = d >= 2 ? Ls + e : e;
            if (fill_R) {
              for (int o = R0; o < cn; o++)
                Rs = COMB(Rs, COMB(XJ(cur, y + o, d) + TSC(v, o), XR(cur, y + o, d) + TSC(v, o)));
              XR(cur, v, d) = Rs;
            }
          }
        }
      } else if (t == CMGB_MR_st || t == CMGB_IR_st) {
        if (!detached) {
          const int L0 = t == CMGB_IR_st ? 1 : 0;
          const SCT ej = ESC(v)[dsq[j]];
          for (int d = 1; d <= dxA[v]; d++) {
            SCT Js = INIT_SC(v, d - 1), Rs = INIT_SC(v, d - 1), Ls = INIT_SC(v, d);
            if (fill_L) XL(cur, v, d) = Ls;
            for (int o = 0; o < cn; o++) {
              Js = COMB(Js, XJ(prv, y + o, d - 1) + TSC(v, o));
              if (fill_R) Rs = COMB(Rs, XR(prv, y + o, d - 1) + TSC(v, o));
            }
            XJ(cur, v, d) = Js + ej;
            if (fill_R) XR(cur, v, d) = d >= 2 ? Rs + ej : ej;
            if (fill_L) {
              for (int o = L0; o < cn; o++)
                Ls = COMB(Ls, COMB(XJ(cur, y + o, d) + TSC(v, o), XL(cur, y + o, d) + TSC(v, o)));
              XL(cur, v, d) = Ls;
            }
          }
        }
      } else if (t == CMGB_MP_st) {
        const SCT rj = RMESC(v)[dsq[j]];
        for (int d = 1; d <= dxA[v]; d++) {
          const int64_t i = j - d + 1;
          SCT Js = d >= 2 ? INIT_SC(v, d - 2) : IMPV, Ls = INIT_SC(v, d - 1), Rs = INIT_SC(v, d - 1);
          for (int o = 0; o < cn; o++) {
            if (d >= 2) Js = COMB(Js, XJ(prv, y + o, d - 2) + TSC(v, o));
            if (fill_L) Ls = COMB(Ls, MAXF(XJ(cur, y + o, d - 1) + TSC(v, o), XL(cur, y + o, d - 1) + TSC(v, o)));
            if (fill_R) Rs = COMB(Rs, MAXF(XJ(prv, y + o, d - 1) + TSC(v, o), XR(prv, y + o, d - 1) + TSC(v, o)));
          }
          XJ(cur, v, d) = d >= 2 ? Js + ESC(v)[dsq[i] * Kp + dsq[j]] : IMPV;
          if (fill_L) XL(cur, v, d) = d >= 2 ? Ls + LMESC(v)[dsq[i]] : LMESC(v)[dsq[i]];
          if (fill_R) XR(cur, v, d) = d >= 2 ? Rs + rj : rj;
        }
      } else {   /* S, D: no emission */
        for (int d = 1; d <= dxA[v]; d++) {
          SCT Js = INIT_SC(v, d), Ls = INIT_SC(v, d), Rs = INIT_SC(v, d);
          for (int o = 0; o < cn; o++) {
            Js = COMB(Js, XJ(cur, y + o, d) + TSC(v, o));
            if (fill_L) Ls = COMB(Ls, XL(cur, y + o, d) + TSC(v, o));
            if (fill_R) Rs = COMB(Rs, XR(cur, y + o, d) + TSC(v, o));
          }
          XJ(cur, v, d) = Js;
          if (fill_L) XL(cur, v, d) = Ls;
          if (fill_R) XR(cur, v, d) = Rs;
        }
      }
      /* per-state best score: a running maximum for CYK, the current row's
       * maximum for integer Inside (src/cm_dpsearch_trunc.c:490-512, 1116-1134) */
      {
        SCT b = IMPV;
        const int begl = m->stid[v] == CMGB_BEGL_S;
        const int r0 = (int) (j % WP);
        for (int d = 1; d <= dxA[v]; d++) {
          b = MAXF(b, begl ? BJ(r0, v, d) : XJ(cur, v, d));
          if (fill_L) b = MAXF(b, begl ? BL(r0, v, d) : XL(cur, v, d));
          if (fill_R) b = MAXF(b, begl ? BR(r0, v, d) : XR(cur, v, d));
          if (t == CMGB_B_st && fill_T) b = MAXF(b, XT(cur, v, d));
        }
#if RUNNING_VSC
        c->vsc[v] = MAXF(c->vsc[v], SCOREF(b));
#else
        c->vsc[v] = SCOREF(b);
#endif
      }
    }

    /* root: truncated begins into every state with a penalty; the root's
     * cells keep the best score seen at this row parity and length
     * (src/cm_dpsearch_trunc.c:540-610, 1178-1250) */
    for (int d = 0; d <= W; d++) { c->bestf[d] = IMP; c->bestr[d] = 0; c->bestmode[d] = CMGB_TRMODE_UNKNOWN; }
    for (int yy = 1; yy < M; yy++) {
      const SCT pen = PTY(yy);
      if (!IS_PTY(pen)) continue;
      const int dx = MINF(dxA[0], dxA[yy]);
      for (int mode = 0; mode < 4; mode++) {
        SCT *X; int code;
        if (mode == 0) { X = Jm; code = CMGB_TRMODE_J; }
        else if (mode == 1) { if (!fill_L) continue; X = Lm; code = CMGB_TRMODE_L; }
        else if (mode == 2) { if (!fill_R) continue; X = Rm; code = CMGB_TRMODE_R; }
        else { if (!(fill_T && m->sttype[yy] == CMGB_B_st)) continue; X = Tm; code = CMGB_TRMODE_T; }
        for (int d = 1; d <= dx; d++) {
          const SCT sc = X[((size_t) cur * M + yy) * WP + d] + pen;
          SCT *root = &X[((size_t) cur * M + 0) * WP + d];
          if (sc > *root) {
            *root = sc;
            const float f = SCOREF(sc);
            if (f > c->bestf[d]) { c->bestf[d] = f; c->bestmode[d] = code; c->bestr[d] = yy; }
          }
        }
      }
    }
    for (int d = 1; d <= dxA[0]; d++)
      if (c->bestf[d] > c->vsc_root) { c->vsc_root = c->bestf[d]; c->vmode_root = c->bestmode[d]; }
    for (int d = 1; d <= dxA[0]; d++)
      if (c->bestf[d] >= c->env_cutoff) { c->envi = MINF(c->envi, j - d + 1); c->envj = MAXF(c->envj, j); }
    report_j(c, j, jp_g, 1, dxA[0]);
  }
#undef XJ
#undef XL
#undef XR
#undef XT
#undef BJ
#undef BL
#undef BR
  free(dxA); free(Jm); free(Lm); free(Rm); free(Tm); free(Jb); free(Lb); free(Rb);
}
#undef TR_CORE_NAME
#undef SCT
#undef IMPV
#undef COMB
#undef IS_PTY
#undef SCOREF
#undef TSC
#undef ESC
#undef LMESC
#undef RMESC
#undef PTY
#undef INIT_SC
#undef ENDSC
#undef RUNNING_VSC
