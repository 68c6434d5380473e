/* cm_scan_oracle_core.h -- typed DP core of the scan oracle (TEST
 * INFRASTRUCTURE ONLY; included three times by cm_scan_oracle.c with the
 * macros CORE_NAME, SCT, IMPV, COMB, ROOTFIRST, SCOREF, ENVF, TSC, ESC,
 * ESCT (emission table element type), EV (emission value as SCT), BEGINSC,
 * HAS_BEGIN, ENDSC, INIT_SC).
 *
 * Restates the j / v / d loops of FastCYKScan (src/cm_dpsearch.c:215-634),
 * FastIInsideScan (:1232-1647) and FastFInsideScan (:1851-2270): rolling
 * rows alpha[j%2][v][d], the BEGL ring alpha_begl[j%(W+1)][v][d], d = 0
 * initialisation (src/cm_mx.c:6039-6138), the Fast scanners' child fold
 * order per child count, root/local begins and per-j hit bookkeeping. */
static void CORE_NAME(scanctx *c)
{
  const cmgb_model_desc *m = c->m;
  const uint8_t *dsq = c->dsq;
  const int M = c->M, Wm = c->Wm, W = c->W, WP = c->WP, Kp = c->Kp, K = c->K;
  const int nb = c->nbegl ? c->nbegl : 1;
  const int *dn = c->dn, *dxW = c->dxW, *beglidx = c->beglidx;
  SCT *alpha = malloc(sizeof(SCT) * 2 * (size_t) M * WP);
  SCT *begl = malloc(sizeof(SCT) * (size_t) (W + 1) * nb * WP);
  SCT *init = malloc(sizeof(SCT) * (size_t) M * WP);
  SCT *bestsc = malloc(sizeof(SCT) * WP);
  for (size_t k = 0; k < 2 * (size_t) M * WP; k++) alpha[k] = IMPV;
  for (size_t k = 0; k < (size_t) (W + 1) * nb * WP; k++) begl[k] = IMPV;
#define A(r, v, d)  alpha[((size_t) (r) * M + (v)) * WP + (d)]
#define BG(r, b, d) begl[((size_t) (r) * nb + (b)) * WP + (d)]
  for (int v = M - 1; v >= 0; v--) {
    int t = m->sttype[v], y = m->cfirst[v];
    SCT x = IMPV;
    if (m->stid[v] == CMGB_BEGL_S || t == CMGB_S_st || t == CMGB_D_st) {
      x = ENDSC(v);
      for (int o = 0; o < m->cnum[v]; o++) { SCT cand = A(0, y + o, 0) + TSC(v, o); x = MAXF(x, cand); }
      x = MAXF(x, IMPV);
    } else if (t == CMGB_E_st) x = 0;
    else if (t == CMGB_B_st) x = BG(0, beglidx[m->cfirst[v]], 0) + A(0, m->cnum[v], 0);
    if (m->stid[v] == CMGB_BEGL_S) { for (int r = 0; r <= W; r++) BG(r, beglidx[v], 0) = x; }
    else { A(0, v, 0) = x; A(1, v, 0) = x; }
  }
  for (int v = 0; v < M; v++) for (int d = 0; d <= Wm; d++) init[(size_t) v * WP + d] = INIT_SC(v, d);
#define INIT(v, d) init[(size_t) (v) * WP + (d)]

  for (int64_t j = c->i0; j <= c->j0; j++) {
    const int64_t jp = j - c->i0 + 1;
    const int cur = (int) (j % 2), prv = (int) ((j - 1) % 2);
    const int jrow = (int) (j % (W + 1));
    const int jr = jp >= W ? W : (int) jp;
    if (c->act) {
      memcpy(c->act[jp % (W + 1)], c->act[(jp - 1) % (W + 1)], sizeof(double[8]));
      count_residue(c->act[jp % (W + 1)], dsq[j], K);
    }
    for (int v = M - 1; v > 0; v--) {
      const int t = m->sttype[v];
      if (t == CMGB_E_st) continue;
      const int sd = st_delta(t), cnum = m->cnum[v], y0 = m->cfirst[v];
      const int dnv = dn[v], dxv = MINF(jr, dxW[v]);
      const int jpy = st_right(t) ? prv : cur;
      const int isbegl = (m->stid[v] == CMGB_BEGL_S);
      const ESCT *esc = (t == CMGB_B_st || t == CMGB_S_st || t == CMGB_D_st) ? NULL : ESC(v);
      SCT tv[MAXC];
      for (int o = 0; o < cnum && o < MAXC; o++) tv[o] = TSC(v, o);
      SCT *out = isbegl ? &BG(jrow, beglidx[v], 0) : &A(cur, v, 0);
      float vbest = c->vsc[v];
      if (t == CMGB_B_st) {
        const int w = m->cfirst[v], yy = m->cnum[v];
        const SCT *ycol = &A(cur, yy, 0);
        for (int d = dnv; d <= dxv; d++) {
          int kmin, kmax;
          if (c->dmin) {
            int dny = MINF(c->dmin[yy], Wm), dxy = MINF(c->dmax[yy], Wm), dnw = MINF(c->dmin[w], Wm), dxw = MINF(c->dmax[w], Wm);
            kmin = MAXF(0, MAXF(dny, d - dxw)); kmax = MINF(dxy, d - dnw);
          } else { kmin = 0; kmax = d; }
          SCT sc = INIT(v, d);
          int br = (int) ((j - kmin) % (W + 1));
          for (int k = kmin; k <= kmax; k++) {
            sc = COMB(sc, BG(br, beglidx[w], d - k) + ycol[k]);
            br = br == 0 ? W : br - 1;
          }
          out[d] = sc;
          float sf = SCOREF(sc); vbest = MAXF(vbest, sf);
        }
      } else if (isbegl) {
        for (int d = dnv; d <= dxv; d++) {
          SCT sc = INIT(v, d);
          for (int o = 0; o < cnum; o++) sc = COMB(sc, A(jpy, y0 + o, d) + tv[o]);
          out[d] = sc;
          float sf = SCOREF(sc); vbest = MAXF(vbest, sf);
        }
      } else {
        const SCT *ch[MAXC];
        for (int o = 0; o < cnum; o++) ch[o] = &A(jpy, y0 + o, 0);
        const SCT *iv = &INIT(v, 0);
        const int em = (t == CMGB_MP_st) ? 3 : st_left(t) ? 1 : st_right(t) ? 2 : 0;
        for (int d = dnv; d <= dxv; d++) {
          const int dp = d - sd;
          SCT sc;
          /* the Fast scanners' fold order per child count (src/cm_dpsearch.c:307-519) */
          switch (cnum) {
          case 2: sc = COMB(ch[1][dp] + tv[1], iv[dp]); sc = COMB(sc, ch[0][dp] + tv[0]); break;
          case 3: sc = COMB(ch[2][dp] + tv[2], ch[1][dp] + tv[1]); sc = COMB(sc, iv[dp]); sc = COMB(sc, ch[0][dp] + tv[0]); break;
          case 4: sc = COMB(ch[3][dp] + tv[3], ch[2][dp] + tv[2]); sc = COMB(sc, iv[dp]); sc = COMB(sc, ch[1][dp] + tv[1]);
                  sc = COMB(sc, ch[0][dp] + tv[0]); break;
          case 5: sc = COMB(ch[4][dp] + tv[4], ch[3][dp] + tv[3]); sc = COMB(sc, iv[dp]); sc = COMB(sc, ch[1][dp] + tv[1]);
                  sc = COMB(sc, ch[2][dp] + tv[2]); sc = COMB(sc, ch[0][dp] + tv[0]); break;
          default: sc = COMB(ch[5][dp] + tv[5], iv[dp]); sc = COMB(sc, ch[4][dp] + tv[4]); sc = COMB(sc, ch[3][dp] + tv[3]);
                   sc = COMB(sc, ch[2][dp] + tv[2]); sc = COMB(sc, ch[1][dp] + tv[1]); sc = COMB(sc, ch[0][dp] + tv[0]); break;
          }
          const int64_t i = j - d + 1;
          if (em == 3) sc += EV(esc[dsq[i] * Kp + dsq[j]]);
          else if (em == 1) sc += EV(esc[dsq[i]]);
          else if (em == 2) sc += EV(esc[dsq[j]]);
          out[d] = sc;   /* IL reads this cell as its own child at d+1 */
          float sf = SCOREF(sc); vbest = MAXF(vbest, sf);
        }
      }
      c->vsc[v] = vbest;
    }
    /* root and local begins (src/cm_dpsearch.c:562-616) */
    const int dn0 = dn[0], dx0 = MINF(jr, dxW[0]);
    for (int d = 0; d <= W; d++) { c->bestr[d] = -1; c->bestf[d] = IMP; }
    SCT *root = &A(cur, 0, 0);
    for (int d = dn0; d <= dx0; d++) {
      c->bestr[d] = 0;
      const int y = m->cfirst[0];
      SCT r = ROOTFIRST(A(cur, y, d) + TSC(0, 0));
      for (int o = 1; o < m->cnum[0]; o++) r = COMB(r, A(cur, y + o, d) + TSC(0, o));
      root[d] = r;
    }
    if (m->flags & CMGB_LOCAL_BEGIN) {
      for (int y = 1; y < M; y++) {
        if (!HAS_BEGIN(y)) continue;
        const int lo = MAXF(dn0, dn[y]), hi = MINF(dx0, MINF(jr, dxW[y]));
        const SCT *col = (m->stid[y] == CMGB_BEGL_S) ? &BG(jrow, beglidx[y], 0) : &A(cur, y, 0);
        const SCT b = BEGINSC(y);
        for (int d = lo; d <= hi; d++) { SCT s = col[d] + b; if (root[d] < s) { root[d] = s; c->bestr[d] = y; } }
      }
    }
    for (int d = dn0; d <= dx0; d++) {
      c->bestf[d] = SCOREF(root[d]);
      c->vsc_root = MAXF(c->vsc_root, c->bestf[d]);
      if (ENVF(root[d]) >= c->env_cutoff) { if (j - d + 1 < c->envi) c->envi = j - d + 1; if (j > c->envj) c->envj = j; }
    }
    if (c->want_hits && dn0 > dx0) { if (c->gamma_mode) { c->gmx[jp] = c->gmx[jp - 1]; c->gback[jp] = -1; } continue; }
    report_j(c, j, jp, dn0, dx0);
  }
  free(alpha); free(begl); free(init); free(bestsc);
#undef A
#undef BG
#undef INIT
}
#undef CORE_NAME
#undef SCT
#undef IMPV
#undef COMB
#undef ROOTFIRST
#undef SCOREF
#undef ENVF
#undef TSC
#undef ESC
#undef ESCT
#undef EV
#undef BEGINSC
#undef HAS_BEGIN
#undef ENDSC
#undef INIT_SC
