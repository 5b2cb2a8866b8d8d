/* Body of oracle/lbm_ref.c, included once per compute type T (float, double). */
#define XCAT(a, b) a##_##b
#define CAT(a, b) XCAT(a, b)
#define FN(name) CAT(name, SFX)

static void FN(macroscopic)(const lattice_t* L, const T* f, T* rho, T* u) {
  T r = (T)0 + f[0];
  for (int l = 1; l < L->q; ++l) r = r + f[l];
  *rho = r;
  for (int d = 0; d < L->d; ++d) {
    T acc = (T)0;
    for (int l = 0; l < L->q; ++l) {
      if (L->c[l][d] == 1) acc = acc + f[l];
      if (L->c[l][d] == -1) acc = acc - f[l];
    }
    u[d] = acc / r;
  }
}

static T FN(usqr)(const lattice_t* L, const T* u) {
  T s = u[0] * u[0];
  for (int d = 1; d < L->d; ++d) s = s + u[d] * u[d];
  return (T)1.5 * s;
}

static T FN(feq_l)(const lattice_t* L, int l, T rho, const T* u, T usqr) {
  T cu = (T)0;
  for (int d = 0; d < L->d; ++d) {
    if (L->c[l][d] == 1) cu = cu + u[d];
    if (L->c[l][d] == -1) cu = cu - u[d];
  }
  cu = cu * (T)3;
  return rho * (T)L->w[l] * ((T)1 + cu * ((T)1 + (T)0.5 * cu) - usqr);
}

static void FN(equilibrium)(const lattice_t* L, T rho, const T* u, T* feq) {
  const T us = FN(usqr)(L, u);
  for (int l = 0; l < L->q; ++l) feq[l] = FN(feq_l)(L, l, rho, u, us);
}

static void FN(second_moment)(const lattice_t* L, const T* fneq, T* pi) {
  for (int t = 0; t < L->nt; ++t) {
    T acc = (T)0;
    for (int q = 0; q < L->q; ++q) {
      if (L->cc[q][t] == 1) acc = acc + fneq[q];
      if (L->cc[q][t] == -1) acc = acc - fneq[q];
    }
    pi[t] = acc;
  }
}

static void FN(kbc)(const lattice_t* L, const T* f, const T* feq, T rho, T omega, T* fo) {
  T fneq[MAXQ], pi[6], ds[MAXQ], dh[MAXQ];
  for (int l = 0; l < L->q; ++l) fneq[l] = f[l] - feq[l];
  FN(second_moment)(L, fneq, pi);
  for (int l = 0; l < L->q; ++l) ds[l] = (T)0;
  const T two = (T)2, four = (T)4, six = (T)6;
  if (L->q == 27) {
    const T nxz = pi[0] - pi[5], nyz = pi[3] - pi[5];
    const T a = (two * nxz - nyz) / six, b = (-nxz + two * nyz) / six, cz = (-nxz - nyz) / six;
    const T p1 = pi[1] / four, p2 = pi[2] / four, p4 = pi[4] / four;
    const T m1 = -pi[1] / four, m2 = -pi[2] / four, m4 = -pi[4] / four;
    ds[9] = a; ds[18] = a; ds[3] = b; ds[6] = b; ds[1] = cz; ds[2] = cz;
    ds[12] = p1; ds[24] = p1; ds[21] = m1; ds[15] = m1;
    ds[10] = p2; ds[20] = p2; ds[19] = m2; ds[11] = m2;
    ds[8] = p4; ds[4] = p4; ds[7] = m4; ds[5] = m4;
    for (int l = 0; l < L->q; ++l) ds[l] = ds[l] * rho;
  } else {
    const T n = pi[0] - pi[2];
    ds[3] = n; ds[6] = n; ds[2] = -n; ds[1] = -n;
    ds[8] = pi[1]; ds[4] = -pi[1]; ds[5] = -pi[1]; ds[7] = pi[1];
    for (int l = 0; l < L->q; ++l) ds[l] = ds[l] * rho / four;
  }
  const T beta = (T)0.5 * omega, inv_beta = (T)1 / beta;
  T sp1 = (T)0, sp2 = (T)0;
  for (int l = 0; l < L->q; ++l) {
    dh[l] = fneq[l] - ds[l];
    const T temp = dh[l] / feq[l];
    sp1 = sp1 + temp * ds[l];
    sp2 = sp2 + temp * dh[l];
  }
  const T gamma = inv_beta - (two - inv_beta) * sp1 / ((T)1e-32 + sp2);
  for (int l = 0; l < L->q; ++l) fo[l] = f[l] - beta * (two * ds[l] + gamma * dh[l]);
}

static void FN(bgk_pair)(const lattice_t* L, const T* f, T omega, T* fo) {
  T rho = f[0], j[3] = {(T)0, (T)0, (T)0}, u[3];
  for (int l = 1; l < L->q; ++l) {
    const int o = L->opp[l];
    if (l >= o) continue;
    const T sig = f[l] + f[o], dif = f[l] - f[o];
    rho = rho + sig;
    for (int d = 0; d < L->d; ++d) {
      if (L->c[l][d] == 1) j[d] = j[d] + dif;
      if (L->c[l][d] == -1) j[d] = j[d] - dif;
    }
  }
  const T inv = (T)1 / rho;
  for (int d = 0; d < L->d; ++d) u[d] = j[d] * inv;
  /* FP32 compute fuses multiply-adds (fmaf, correctly rounded), as the CUDA path does */
  const int fused = sizeof(T) == 4;
  T usq = u[0] * u[0];
  for (int d = 1; d < L->d; ++d) usq = fused ? (T)fmaf((float)u[d], (float)u[d], (float)usq) : usq + u[d] * u[d];
  const T base = fused ? (T)fmaf(-1.5f, (float)usq, 1.0f) : (T)1 - (T)1.5 * usq;
  const T omf = (T)1 - omega, orho = omega * rho;
  const T r0 = orho * (T)L->w[0] * base;
  fo[0] = fused ? (T)fmaf((float)omf, (float)f[0], (float)r0) : omf * f[0] + r0;
  for (int l = 1; l < L->q; ++l) {
    const int o = L->opp[l];
    if (l >= o) continue;
    T cu = (T)0;
    for (int d = 0; d < L->d; ++d) {
      if (L->c[l][d] == 1) cu = cu + u[d];
      if (L->c[l][d] == -1) cu = cu - u[d];
    }
    const T t = (T)3 * cu, ow = orho * (T)L->w[l];
    if (fused) {
      const T h = (T)4.5 * cu;
      const T e = (T)fmaf((float)h, (float)cu, (float)base);
      const T pl = ow * (e + t), po = ow * (e - t);
      fo[l] = (T)fmaf((float)omf, (float)f[l], (float)pl);
      fo[o] = (T)fmaf((float)omf, (float)f[o], (float)po);
    } else {
      const T e = base + (T)4.5 * (cu * cu);
      fo[l] = omf * f[l] + ow * (e + t);
      fo[o] = omf * f[o] + ow * (e - t);
    }
  }
}

static void FN(normal)(const lattice_t* L, uint32_t miss, int* nv) {
  for (int d = 0; d < L->d; ++d) nv[d] = 0;
  for (int l = 0; l < L->q; ++l) {
    int n1 = 0;
    for (int d = 0; d < L->d; ++d) n1 += abs(L->c[l][d]);
    if (n1 == 1 && ((miss >> l) & 1u)) {
      for (int d = 0; d < L->d; ++d) nv[d] = -L->c[l][d];
      return;
    }
  }
}

static void FN(zouhe_like)(const lattice_t* L, T* f, uint32_t miss, T aux, int kind) {
  int nv[3];
  FN(normal)(L, miss, nv);
  T known = (T)0, middle = (T)0;
  for (int l = 0; l < L->q; ++l) {
    const int k = (miss >> L->opp[l]) & 1u;
    const int m = !k && !((miss >> l) & 1u);
    if (k) known = known + (T)2 * f[l];
    if (m) middle = middle + f[l];
  }
  const T fsum = known + middle;
  T rho, u[3];
  if (kind == BC_ZOUHE_V || kind == BC_REG_V) {
    T un = (T)0;
    for (int d = 0; d < L->d; ++d) u[d] = (-aux) * (T)nv[d];
    for (int d = 0; d < L->d; ++d) un = un + u[d] * (T)nv[d];
    rho = fsum / ((T)1 + un);
  } else {
    rho = aux;
    const T un = (T)-1 + fsum / rho;
    for (int d = 0; d < L->d; ++d) u[d] = un * (T)nv[d];
  }
  T feq[MAXQ];
  FN(equilibrium)(L, rho, u, feq);
  for (int l = 0; l < L->q; ++l)
    if ((miss >> l) & 1u) f[l] = f[L->opp[l]] + feq[l] - feq[L->opp[l]];
  if (kind == BC_REG_V || kind == BC_REG_P) {
    T fneq[MAXQ], pi[6];
    for (int l = 0; l < L->q; ++l) fneq[l] = f[l] - feq[l];
    FN(second_moment)(L, fneq, pi);
    for (int l = 0; l < L->q; ++l) {
      T acc = (T)0;
      for (int t = 0; t < L->nt; ++t)
        if (L->qi[l][t] != 0.0) acc = acc + (T)L->qi[l][t] * pi[t];
      f[l] = feq[l] + (T)4.5 * (T)L->w[l] * acc;
    }
  }
}

static inline int FN(wrap)(int i, int n) { return i < 0 ? n - 1 : (i >= n ? 0 : i); }

/*
 * XLB-order BGK (collision 0) on a chunk of nk <= FLUID_W fluid cells z .. z+nk-1
 * of one row, 1 <= z and z + nk <= n2 - 1 (no wrap along the contiguous
 * axis).  Every cell gets exactly the per-cell operations of the generic path
 * (macroscopic, equilibrium, f - omega (f - feq), in the same order); the loops
 * run over the chunk's cells innermost so the compiler can vectorise them.
 * Speed only: results are bit-identical to the per-cell path.
 */
#ifndef FLUID_W
#define FLUID_W 256
#endif
static void FN(fluid_chunk)(const lattice_t* L, const T* f0, T* f1, int64_t N, const int64_t* src_row,
                            int64_t cell0, int z, int nk, T omega) {
  const int Q = L->q;
  T F[MAXQ][FLUID_W], R[FLUID_W], U[3][FLUID_W], US[FLUID_W];
  for (int l = 0; l < Q; ++l) {
    const T* src = f0 + src_row[l] + z - L->ax[l][2];
    for (int k = 0; k < nk; ++k) F[l][k] = src[k];
  }
  for (int k = 0; k < nk; ++k) R[k] = (T)0 + F[0][k];
  for (int l = 1; l < Q; ++l)
    for (int k = 0; k < nk; ++k) R[k] = R[k] + F[l][k];
  for (int d = 0; d < L->d; ++d) {
    T acc[FLUID_W];
    for (int k = 0; k < nk; ++k) acc[k] = (T)0;
    for (int l = 0; l < Q; ++l) {
      if (L->c[l][d] == 1)
        for (int k = 0; k < nk; ++k) acc[k] = acc[k] + F[l][k];
      if (L->c[l][d] == -1)
        for (int k = 0; k < nk; ++k) acc[k] = acc[k] - F[l][k];
    }
    for (int k = 0; k < nk; ++k) U[d][k] = acc[k] / R[k];
  }
  for (int k = 0; k < nk; ++k) US[k] = U[0][k] * U[0][k];
  for (int d = 1; d < L->d; ++d)
    for (int k = 0; k < nk; ++k) US[k] = US[k] + U[d][k] * U[d][k];
  for (int k = 0; k < nk; ++k) US[k] = (T)1.5 * US[k];
  for (int l = 0; l < Q; ++l) {
    const T w = (T)L->w[l];
    T cu[FLUID_W];
    for (int k = 0; k < nk; ++k) cu[k] = (T)0;
    for (int d = 0; d < L->d; ++d) {
      if (L->c[l][d] == 1)
        for (int k = 0; k < nk; ++k) cu[k] = cu[k] + U[d][k];
      if (L->c[l][d] == -1)
        for (int k = 0; k < nk; ++k) cu[k] = cu[k] - U[d][k];
    }
    T* dst = f1 + (int64_t)l * N + cell0;
    for (int k = 0; k < nk; ++k) {
      const T c3 = cu[k] * (T)3;
      const T feq = R[k] * w * ((T)1 + c3 * ((T)1 + (T)0.5 * c3) - US[k]);
      dst[k] = F[l][k] - omega * (F[l][k] - feq);
    }
  }
}

/*
 * One step.  f0 is read (and receives the aux recovery writes afterwards), f1 is
 * written.  Per-BC arrays: ids, kinds, rhos, us (3 per BC).  Returns 0.
 */
int FN(lbm_ref_step)(int lattice, int collision, int64_t nx, int64_t ny, int64_t nz, T* f0, T* f1,
                     const uint8_t* bcm, const uint32_t* miss, int nbc, const int* ids, const int* kinds,
                     const double* rhos, const double* us, double omega_d, int nthreads) {
  lattice_t Ls;
  make_lattice(lattice, &Ls);
  const lattice_t* L = &Ls;
  const int n0 = lattice == 0 ? 1 : (int)nx, n1 = lattice == 0 ? (int)nx : (int)ny, n2 = lattice == 0 ? (int)ny : (int)nz;
  const int64_t N = (int64_t)n0 * n1 * n2;
  int kind_of[256] = {0}, slot_of[256];
  for (int b = 0; b < nbc; ++b) {
    kind_of[ids[b]] = kinds[b];
    slot_of[ids[b]] = b;
  }
  const int Q = L->q;
  const T omega = (T)omega_d;
  const T cs = (T)(1.0 / (double)sqrtf(3.0f));
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  /* aux recovery source values: f1 slots at ZouHe / Regularized cells, before the step writes f1 */
  int64_t nrec = 0;
  for (int64_t c = 0; c < N; ++c) {
    const int k = kind_of[bcm[c]];
    if (bcm[c] != 255 && k >= BC_ZOUHE_V && k <= BC_REG_P) ++nrec;
  }
  int64_t* rec = nrec ? (int64_t*)malloc(sizeof(int64_t) * nrec) : NULL;
  T* sav = nrec ? (T*)malloc(sizeof(T) * nrec * Q) : NULL;
  {
    int64_t r = 0;
    for (int64_t c = 0; c < N; ++c) {
      const int k = kind_of[bcm[c]];
      if (bcm[c] != 255 && k >= BC_ZOUHE_V && k <= BC_REG_P) {
        rec[r] = c;
        for (int l = 0; l < Q; ++l) sav[r * Q + l] = f1[(int64_t)l * N + c];
        ++r;
      }
    }
  }

#pragma omp parallel for schedule(static)
  for (int64_t row = 0; row < (int64_t)n0 * n1; ++row) {
    const int i0 = (int)(row / n1), i1 = (int)(row % n1);
    int64_t src_row[MAXQ];
    for (int l = 0; l < Q; ++l)
      src_row[l] = (int64_t)l * N +
                   ((int64_t)FN(wrap)(i0 - L->ax[l][0], n0) * n1 + FN(wrap)(i1 - L->ax[l][1], n1)) * n2;
    for (int i2 = 0; i2 < n2; ++i2) {
      const int64_t cell = row * n2 + i2;
      if (collision == 0 && i2 >= 1 && i2 < n2 - 1) {
        const int nk = n2 - 1 - i2 < FLUID_W ? n2 - 1 - i2 : FLUID_W;
        int fluid = 1;
        for (int k = 0; k < nk; ++k) fluid &= bcm[cell + k] == 0;
        if (fluid) {
          FN(fluid_chunk)(L, f0, f1, N, src_row, cell, i2, nk, omega);
          i2 += nk - 1;
          continue;
        }
      }
      const uint8_t id = bcm[cell];
      if (id == 255) continue;
      T f[MAXQ], fo[MAXQ], feq[MAXQ], u[3], rho;
      for (int l = 0; l < Q; ++l) {
        const int s0 = FN(wrap)(i0 - L->ax[l][0], n0), s1 = FN(wrap)(i1 - L->ax[l][1], n1), s2 = FN(wrap)(i2 - L->ax[l][2], n2);
        f[l] = f0[(int64_t)l * N + ((int64_t)s0 * n1 + s1) * n2 + s2];
      }
      const int kind = id ? kind_of[id] : 0;
      const uint32_t m = id ? miss[cell] : 0u;
      if (kind == BC_HALFWAY || kind == BC_EXTRAP) {
        for (int l = 0; l < Q; ++l)
          if ((m >> l) & 1u) f[l] = f0[(int64_t)L->opp[l] * N + cell];
      } else if (kind == BC_EQUILIBRIUM) {
        const int b = slot_of[id];
        T ub[3];
        for (int d = 0; d < L->d; ++d) ub[d] = (T)us[3 * b + d];
        FN(equilibrium)(L, (T)rhos[b], ub, f);
      } else if (kind >= BC_ZOUHE_V && kind <= BC_REG_P) {
        FN(zouhe_like)(L, f, m, f1[cell], kind);
      }
      if (collision == 2) {
        FN(bgk_pair)(L, f, omega, fo);
      } else {
        FN(macroscopic)(L, f, &rho, u);
        FN(equilibrium)(L, rho, u, feq);
        if (collision == 0) {
          for (int l = 0; l < Q; ++l) fo[l] = f[l] - omega * (f[l] - feq[l]);
        } else {
          FN(kbc)(L, f, feq, rho, omega, fo);
        }
      }
      if (kind == BC_FULLWAY) {
        for (int l = 0; l < Q; ++l) fo[l] = f[L->opp[l]];
      } else if (kind == BC_EXTRAP) {
        int nv[3], ii[3] = {i0, i1, i2}, nn[3] = {n0, n1, n2};
        FN(normal)(L, m, nv);
        for (int l = 0; l < Q; ++l) {
          if (!((m >> l) & 1u)) continue;
          int s[3];
          for (int k = 0; k < 3; ++k) {
            const int off = L->ax[l][k] + (L->d == 3 ? nv[k] : (k == 0 ? 0 : nv[k - 1]));
            int v = (ii[k] - off) % nn[k];
            s[k] = v < 0 ? v + nn[k] : v;
          }
          const T faux = f0[(int64_t)l * N + ((int64_t)s[0] * n1 + s[1]) * n2 + s[2]];
          fo[L->opp[l]] = ((T)1 - cs) * f[l] + cs * faux;
        }
      }
      for (int l = 0; l < Q; ++l) f1[(int64_t)l * N + cell] = fo[l];
    }
  }

  for (int64_t r = 0; r < nrec; ++r) {
    const int64_t c = rec[r];
    const uint32_t m = miss[c];
    f0[c] = sav[r * Q];
    for (int l = 1; l < Q; ++l)
      if ((m >> l) & 1u) f0[(int64_t)L->opp[l] * N + c] = sav[r * Q + L->opp[l]];
  }
  free(rec);
  free(sav);
  return 0;
}

#undef FN
#undef CAT
#undef XCAT
