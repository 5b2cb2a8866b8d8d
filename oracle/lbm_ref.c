/*
 * lbm_ref.c -- C restatement of XLB's fused stepper.  TEST INFRASTRUCTURE ONLY:
 * used by tests/ as a checker at sizes the numpy oracle is too slow for, and by
 * bench.py as the timed CPU baseline.  Nothing in xlb_gb300 links it.
 *
 * Same semantics and floating-point operation order as oracle/lbm_oracle.py
 * (which cites the XLB source line by line); compile with -ffp-contract=off so
 * no multiply-add is fused.  Store type == compute type (FP32FP32 or FP64FP64).
 *
 * Per cell (xlb/operator/stepper/nse_stepper.py:344-382): skip id 255, pull with
 * a one-cell wrap, streaming-step BC, rho/u, feq, BGK or KBC, collision-step BC
 * and extrapolation aux data, store.  Aux recovery into f0 runs after the whole
 * grid has been updated.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXQ 27

enum { BC_FULLWAY = 1, BC_HALFWAY, BC_EQUILIBRIUM, BC_ZOUHE_V, BC_ZOUHE_P, BC_REG_V, BC_REG_P, BC_EXTRAP };

typedef struct {
  int q, d, nt;
  int c[MAXQ][3];  /* physical components, d used */
  int ax[MAXQ][3]; /* offsets along internal axes (2D embeds as (0, cx, cy)) */
  double w[MAXQ];
  int opp[MAXQ];
  int cc[MAXQ][6];
  double qi[MAXQ][6];
} lattice_t;

static int tri(int digit) { return digit == 0 ? 0 : (digit == 1 ? -1 : 1); }

static void make_lattice(int code, lattice_t* L) {
  memset(L, 0, sizeof(*L));
  if (code == 0) {
    static const int cx[9] = {0, 0, 0, 1, -1, 1, -1, 1, -1}, cy[9] = {0, 1, -1, 0, 1, -1, 0, 1, -1};
    L->q = 9;
    L->d = 2;
    for (int l = 0; l < 9; ++l) {
      L->c[l][0] = cx[l];
      L->c[l][1] = cy[l];
    }
  } else {
    int k = 0;
    for (int l = 0; l < 27; ++l) {
      int v[3] = {tri(l / 9), tri((l / 3) % 3), tri(l % 3)};
      int n1 = abs(v[0]) + abs(v[1]) + abs(v[2]);
      if (code == 1 && n1 > 2) continue;
      for (int a = 0; a < 3; ++a) L->c[k][a] = v[a];
      ++k;
    }
    L->q = k;
    L->d = 3;
  }
  L->nt = L->d * (L->d + 1) / 2;
  for (int l = 0; l < L->q; ++l) {
    int n1 = 0;
    for (int a = 0; a < L->d; ++a) n1 += abs(L->c[l][a]);
    if (L->q == 9)
      L->w[l] = n1 == 0 ? 4.0 / 9.0 : (n1 == 1 ? 1.0 / 9.0 : 1.0 / 36.0);
    else if (L->q == 19)
      L->w[l] = n1 == 0 ? 1.0 / 3.0 : (n1 == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
    else
      L->w[l] = n1 == 0 ? 8.0 / 27.0 : (n1 == 1 ? 2.0 / 27.0 : (n1 == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
    for (int a = 0; a < 3; ++a) L->ax[l][a] = L->d == 3 ? L->c[l][a] : (a == 0 ? 0 : L->c[l][a - 1]);
    int t = 0;
    for (int a = 0; a < L->d; ++a)
      for (int b = a; b < L->d; ++b) {
        L->cc[l][t] = L->c[l][a] * L->c[l][b];
        L->qi[l][t] = a == b ? (double)L->cc[l][t] + (-1.0 / 3.0) : 2.0 * (double)L->cc[l][t];
        ++t;
      }
  }
  for (int l = 0; l < L->q; ++l)
    for (int m = 0; m < L->q; ++m) {
      int same = 1;
      for (int a = 0; a < L->d; ++a) same &= L->c[m][a] == -L->c[l][a];
      if (same) L->opp[l] = m;
    }
}

typedef struct {
  int id, kind;
  double rho, u[3];
} bc_t;

#define T float
#define SFX f32
#include "lbm_ref_body.h"
#undef T
#undef SFX

#define T double
#define SFX f64
#include "lbm_ref_body.h"
#undef T
#undef SFX

int lbm_ref_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
