// Per-cell physics: moments, equilibrium, BGK, KBC and the boundary functionals.
//
// Each function keeps the operation order of the XLB functional it replaces so
// that, built with --fmad=false, results match the CPU oracle bit for bit.
#pragma once
#include "lattice.cuh"

namespace xlbg {

// rho = sum_l f_l ; u_d = (sum_{c_dl=+1} f_l - sum_{c_dl=-1} f_l) / rho
// (zero_moment.py:137-141, first_moment.py:188-201)
template <class L, class T>
__device__ __forceinline__ void macroscopic(const T (&f)[L::Q], T& rho, T (&u)[L::D]) {
  rho = T(0) + f[0];
#pragma unroll
  for (int l = 1; l < L::Q; ++l) rho = rho + f[l];
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    T acc = T(0);
#pragma unroll
    for (int l = 0; l < L::Q; ++l) {
      if (L::c(l, d) == 1) acc = acc + f[l];
      if (L::c(l, d) == -1) acc = acc - f[l];
    }
    u[d] = acc / rho;
  }
}

// feq_l = rho w_l (1 + cu (1 + cu/2) - 1.5 |u|^2), cu = 3 c_l.u (quadratic_equilibrium.py:331-356)
template <class L, class T>
__device__ __forceinline__ T feq_l(int l, T rho, const T (&u)[L::D], T usqr) {
  T cu = T(0);
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    if (L::c(l, d) == 1) cu = cu + u[d];
    if (L::c(l, d) == -1) cu = cu - u[d];
  }
  cu = cu * T(3);
  return rho * T(weight<L>(l)) * (T(1) + cu * (T(1) + T(0.5) * cu) - usqr);
}

template <class L, class T>
__device__ __forceinline__ T usqr_of(const T (&u)[L::D]) {
  T s = u[0] * u[0];
#pragma unroll
  for (int d = 1; d < L::D; ++d) s = s + u[d] * u[d];
  return T(1.5) * s;
}

template <class L, class T>
__device__ __forceinline__ void equilibrium(T rho, const T (&u)[L::D], T (&feq)[L::Q]) {
  const T usqr = usqr_of<L>(u);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) feq[l] = feq_l<L>(l, rho, u, usqr);
}

// Pi_t = sum_q cc_qt fneq_q, with cc in {-1, 0, 1} (second_moment.py:416-426)
template <class L, class T>
__device__ __forceinline__ void second_moment(const T (&fneq)[L::Q], T (&pi)[L::NT]) {
#pragma unroll
  for (int t = 0; t < L::NT; ++t) {
    T acc = T(0);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      if (cc<L>(q, t) == 1) acc = acc + fneq[q];
      if (cc<L>(q, t) == -1) acc = acc - fneq[q];
    }
    pi[t] = acc;
  }
}

// Entropic KBC (kbc.py:192-296); defined for D2Q9 and D3Q27 only.
template <class L, class T>
__device__ __forceinline__ void kbc(const T (&f)[L::Q], const T (&feq)[L::Q], T rho, T omega, T (&fo)[L::Q]) {
  T fneq[L::Q];
#pragma unroll
  for (int l = 0; l < L::Q; ++l) fneq[l] = f[l] - feq[l];
  T pi[L::NT];
  second_moment<L>(fneq, pi);
  T ds[L::Q];
#pragma unroll
  for (int l = 0; l < L::Q; ++l) ds[l] = T(0);
  const T two = T(2), four = T(4), six = T(6);
  if constexpr (L::Q == 27) {
    const T nxz = pi[0] - pi[5];
    const T nyz = pi[3] - pi[5];
    const T a = (two * nxz - nyz) / six;
    const T b = (-nxz + two * nyz) / six;
    const T cz = (-nxz - nyz) / six;
    const T p1 = pi[1] / four, p2 = pi[2] / four, p4 = pi[4] / four;
    const T m1 = -pi[1] / four, m2 = -pi[2] / four, m4 = -pi[4] / four;
    ds[9] = a; ds[18] = a; ds[3] = b; ds[6] = b; ds[1] = cz; ds[2] = cz;
    ds[12] = p1; ds[24] = p1; ds[21] = m1; ds[15] = m1;
    ds[10] = p2; ds[20] = p2; ds[19] = m2; ds[11] = m2;
    ds[8] = p4; ds[4] = p4; ds[7] = m4; ds[5] = m4;
#pragma unroll
    for (int l = 0; l < L::Q; ++l) ds[l] = ds[l] * rho;
  } else {
    const T n = pi[0] - pi[2];
    ds[3] = n; ds[6] = n; ds[2] = -n; ds[1] = -n;
    ds[8] = pi[1]; ds[4] = -pi[1]; ds[5] = -pi[1]; ds[7] = pi[1];
#pragma unroll
    for (int l = 0; l < L::Q; ++l) ds[l] = ds[l] * rho / four;
  }
  const T beta = T(0.5) * omega;
  const T inv_beta = T(1) / beta;
  T dh[L::Q];
  T sp1 = T(0), sp2 = T(0);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    dh[l] = fneq[l] - ds[l];
    // dh / feq, with feq > 0: a zero dh (cells still at their initial equilibrium)
    // is its own quotient, sign included, and skips the division's slow path,
    // which every zero dividend took
    const T temp = dh[l] == T(0) ? dh[l] : dh[l] / feq[l];
    sp1 = sp1 + temp * ds[l];
    sp2 = sp2 + temp * dh[l];
  }
  const T gamma = inv_beta - (two - inv_beta) * sp1 / (T(1e-32) + sp2);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) fo[l] = f[l] - beta * (two * ds[l] + gamma * dh[l]);
}

// BGK in pair form (collision code 2): the same equations as macroscopic +
// quadratic equilibrium + BGK, arranged over opposite-direction pairs (l, opp l)
// with l < opp l.  rho and j come from the pair sums and differences, u = j / rho
// uses one reciprocal, feq of a pair shares e = 1 - 1.5|u|^2 + 4.5 (c.u)^2 and
// t = 3 c.u, and the update is f_out = (1 - omega) f + (omega rho w) (e +- t).
// About 190 floating-point operations per D3Q19 cell instead of about 325
// (about 160 with FP32 compute, which fuses multiply-adds where listed below);
// results differ from XLB's operation order by rounding only.
template <class L>
__host__ __device__ constexpr bool pair_lead(int l) {
  return l != 0 && l < opp<L>(l);
}

// The p-th pair lead (pairs ordered by increasing l).
template <class L>
__host__ __device__ constexpr int pair_at(int p) {
  int k = 0;
  for (int l = 1; l < L::Q; ++l) {
    if (pair_lead<L>(l)) {
      if (k == p) return l;
      ++k;
    }
  }
  return -1;
}

// Recursion over pairs so every index is a compile-time constant.
template <class L, class T, int P>
__device__ __forceinline__ void pair_moments(const T (&f)[L::Q], T& rho, T (&j)[L::D]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    const T sig = f[l] + f[o];
    const T dif = f[l] - f[o];
    rho = rho + sig;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) j[d] = j[d] + dif;
      if (L::c(l, d) == -1) j[d] = j[d] - dif;
    }
    pair_moments<L, T, P + 1>(f, rho, j);
  }
}

template <class L, class T, int P>
__device__ __forceinline__ void pair_update(const T (&f)[L::Q], const T (&u)[L::D], T base, T omf, T orho,
                                            T (&fo)[L::Q]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    T cu = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) cu = cu + u[d];
      if (L::c(l, d) == -1) cu = cu - u[d];
    }
    const T t = T(3) * cu;
    const T ow = orho * T(weight<L>(l));
    if constexpr (sizeof(T) == 4) {
      // FP32: fused multiply-adds (the oracle reproduces them exactly)
      const T e = __fmaf_rn(T(4.5) * cu, cu, base);
      fo[l] = __fmaf_rn(omf, f[l], ow * (e + t));
      fo[o] = __fmaf_rn(omf, f[o], ow * (e - t));
    } else {
      const T e = base + T(4.5) * (cu * cu);
      fo[l] = omf * f[l] + ow * (e + t);
      fo[o] = omf * f[o] + ow * (e - t);
    }
    pair_update<L, T, P + 1>(f, u, base, omf, orho, fo);
  }
}

template <class L, class T>
__device__ __forceinline__ void bgk_pair(const T (&f)[L::Q], T omega, T (&fo)[L::Q]) {
  T rho = f[0];
  T j[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) j[d] = T(0);
  pair_moments<L, T, 0>(f, rho, j);
  const T inv = T(1) / rho;
  T u[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) u[d] = j[d] * inv;
  T usq = u[0] * u[0];
  T base;
  const T omf = T(1) - omega;
  const T orho = omega * rho;
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int d = 1; d < L::D; ++d) usq = __fmaf_rn(u[d], u[d], usq);
    base = __fmaf_rn(T(-1.5), usq, T(1));
    fo[0] = __fmaf_rn(omf, f[0], orho * T(weight<L>(0)) * base);
  } else {
#pragma unroll
    for (int d = 1; d < L::D; ++d) usq = usq + u[d] * u[d];
    base = T(1) - T(1.5) * usq;
    fo[0] = omf * f[0] + orho * T(weight<L>(0)) * base;
  }
  pair_update<L, T, 0>(f, u, base, omf, orho, fo);
}

// BGK on the stored deviations of the shifted FP16 / BF16 forms, and on
// g = f - w for FP32 storage (collision code 3; no XLB counterpart).  The same equations as macroscopic + quadratic
// equilibrium + BGK (bgk.py:30-34, quadratic_equilibrium.py:35-60), written
// for g_l = S (f_l - w_l) as the store holds it (S = 2^14 for FP16S, 1 for
// BF16S) so that a pulled value is one conversion from its bits and a result
// one conversion to them, and no FP32 rounding of f ~ w is paid on top of the
// 16-bit one:
//   rho = 1 + G / S,  u = J / (S rho),   G = sum_l g_l,  J = sum_l c_l g_l,
//   S (feq_l - w_l) = S w_l (rho e_l - 1),  e_l = 1 + t + t^2 / 2 - 1.5 |u|^2,  t = 3 c_l.u,
//   g_out = (1 - omega) g + omega S (feq - w).
// Over an opposite pair (l, o) t changes sign; with A = omega S w (one per
// weight class, carried in two floats), v = 3u, base = 1 - |v|^2 / 6,
// C = A (rho base - 1) and R = C + (A rho / 2) t^2:
//   g_out_l = fma(1 - omega, g_l, fma( A rho, t, R)),
//   g_out_o = fma(1 - omega, g_o, fma(-A rho, t, R)).
// About 125 floating-point operations per D3Q19 cell, decode and encode
// included, against about 200 for the pair form on f.
template <int SK>
__host__ __device__ constexpr float shift_scale() {
  return SK == 3 ? 16384.0f : 1.0f;  // SK_F16S : SK_BF16S and SK_F32 (g = f - w)
}

template <class L, int P>
__device__ __forceinline__ void shifted_pair_update(const float (&g)[L::Q], const float (&v)[L::D],
                                                    const float (&Ar)[4], const float (&Arh)[4], const float (&C)[4],
                                                    float omf, float (&go)[L::Q]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    constexpr int k = norm1<L>(l);
    float t = 0.0f;
    bool first = true;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) != 0) {
        const float x = L::c(l, d) == 1 ? v[d] : -v[d];
        t = first ? x : t + x;
        first = false;
      }
    }
    const float q = Arh[k] * t;
    const float R = __fmaf_rn(q, t, C[k]);
    go[l] = __fmaf_rn(omf, g[l], __fmaf_rn(Ar[k], t, R));
    go[o] = __fmaf_rn(omf, g[o], __fmaf_rn(-Ar[k], t, R));
    shifted_pair_update<L, P + 1>(g, v, Ar, Arh, C, omf, go);
  }
}

template <class L, int SK>
__device__ __forceinline__ void bgk_shifted(const float (&g)[L::Q], float omega, float (&go)[L::Q]) {
  constexpr float S = shift_scale<SK>();
  constexpr float K = 1.0f / S;  // a power of two: exact
  float G = g[0];
  float J[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) J[d] = 0.0f;
  pair_moments<L, float, 0>(g, G, J);
  const float rho = __fmaf_rn(K, G, 1.0f);
  const float k3 = 3.0f * (K * __frcp_rn(rho));
  float v[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) v[d] = J[d] * k3;
  float vsq = v[0] * v[0];
#pragma unroll
  for (int d = 1; d < L::D; ++d) vsq = __fmaf_rn(v[d], v[d], vsq);
  // rho base - 1 = (1 + G/S)(1 + bm1) - 1 = (G/S) base + bm1, bm1 = -|v|^2/6: no
  // cancellation against the 1 of rho or of base
  const float bm1 = (-1.0f / 6.0f) * vsq;
  const float base = 1.0f + bm1;
  const float r = __fmaf_rn(K * G, base, bm1);
  const float omf = 1.0f - omega;
  float Ar[4] = {0.0f, 0.0f, 0.0f, 0.0f}, Arh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, C[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  // S w_k as a float pair hi + lo (compile-time constants; class_weight called with
  // the unrolled index below would not be a constant expression and ran as a loop)
  constexpr double Sw[4] = {(double)S * class_weight<L>(0), (double)S * class_weight<L>(1),
                            (double)S * class_weight<L>(2), (double)S * class_weight<L>(3)};
  constexpr float Whi[4] = {(float)Sw[0], (float)Sw[1], (float)Sw[2], (float)Sw[3]};
  constexpr float Wlo[4] = {(float)(Sw[0] - (double)Whi[0]), (float)(Sw[1] - (double)Whi[1]),
                            (float)(Sw[2] - (double)Whi[2]), (float)(Sw[3] - (double)Whi[3])};
#pragma unroll
  for (int k = 0; k <= L::D; ++k) {
    // weight class |c|_1 = k (D2Q9 and D3Q19 have no k = 3; the unused entries fold away).
    // A = omega S w_k is carried as hi + lo: a rounded A is the same relative error
    // in every cell and step of a class, which breaks the collision's exact
    // momentum and mass balance and accumulates; A rho and A r are each rounded once.
    const float Ahi = omega * Whi[k];
    const float Alo = __fmaf_rn(omega, Whi[k], -Ahi) + omega * Wlo[k];
    Ar[k] = __fmaf_rn(Ahi, rho, Alo * rho);
    Arh[k] = 0.5f * Ar[k];
    C[k] = __fmaf_rn(Ahi, r, Alo * r);
  }
  go[0] = __fmaf_rn(omf, g[0], C[0]);
  shifted_pair_update<L, 0>(g, v, Ar, Arh, C, omf, go);
}

// -c of the first missing direction with |c|_1 = 1 (helper_functions_bc.py:250-261,
// bc_extrapolation_outflow.py:358-369).  Zero when there is none.
template <class L>
__device__ __forceinline__ void normal_of(uint32_t miss, int (&nv)[L::D]) {
  bool found = false;
#pragma unroll
  for (int d = 0; d < L::D; ++d) nv[d] = 0;
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    if (norm1<L>(l) == 1) {
      if (!found && ((miss >> l) & 1u)) {
        found = true;
#pragma unroll
        for (int d = 0; d < L::D; ++d) nv[d] = -L::c(l, d);
      }
    }
  }
}

// BC kinds (include/xlbg.h)
enum {
  BC_FULLWAY = 1,
  BC_HALFWAY = 2,
  BC_EQUILIBRIUM = 3,
  BC_ZOUHE_V = 4,
  BC_ZOUHE_P = 5,
  BC_REG_V = 6,
  BC_REG_P = 7,
  BC_EXTRAP = 8
};

// ZouHe and Regularized, velocity or pressure (bc_zouhe.py:279-343,
// bc_regularized.py:134-202, helpers helper_functions_bc.py:236-297).
template <class L, class T>
__device__ __forceinline__ void zouhe_like(T (&f)[L::Q], uint32_t miss, T aux, int kind) {
  int nv[L::D];
  normal_of<L>(miss, nv);
  T known = T(0), middle = T(0);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    const bool k = (miss >> opp<L>(l)) & 1u;
    const bool m = !k && !((miss >> l) & 1u);
    if (k) known = known + T(2) * f[l];
    if (m) middle = middle + f[l];
  }
  const T fsum = known + middle;
  T rho, u[L::D];
  if (kind == BC_ZOUHE_V || kind == BC_REG_V) {
    T unormal = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = (-aux) * T(nv[d]);
#pragma unroll
    for (int d = 0; d < L::D; ++d) unormal = unormal + u[d] * T(nv[d]);
    rho = fsum / (T(1) + unormal);
  } else {
    rho = aux;
    const T unormal = T(-1) + fsum / rho;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = unormal * T(nv[d]);
  }
  T feq[L::Q];
  equilibrium<L>(rho, u, feq);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    if ((miss >> l) & 1u) f[l] = f[opp<L>(l)] + feq[l] - feq[opp<L>(l)];
  }
  if (kind == BC_REG_V || kind == BC_REG_P) {
    T fneq[L::Q];
#pragma unroll
    for (int l = 0; l < L::Q; ++l) fneq[l] = f[l] - feq[l];
    T pi[L::NT];
    second_moment<L>(fneq, pi);
#pragma unroll
    for (int l = 0; l < L::Q; ++l) {
      T acc = T(0);
#pragma unroll
      for (int t = 0; t < L::NT; ++t) {
        if (qi<L>(l, t) != 0.0) acc = acc + T(qi<L>(l, t)) * pi[t];
      }
      f[l] = feq[l] + T(4.5) * T(weight<L>(l)) * acc;
    }
  }
}

// The boundary functionals on stored deviations g = S (f - w) (collision code 3;
// no XLB counterpart, the equations of quadratic_equilibrium.py:35-60,
// bc_equilibrium.py:75-86 and helper_functions_bc.py:236-297 rewritten so that
// rho - 1 and feq - w are formed without cancellation against 1 or w).
//
// Quadratic equilibrium as deviations: S (feq_l - w_l) = S w_l (rho e_l - 1) with
// rho e_l - 1 = drho e_l + (e_l - 1), e_l - 1 = t + t^2/2 - 1.5 |u|^2, t = 3 c_l.u.
template <class L, int SK>
__device__ __forceinline__ void equilibrium_dev(float drho, const float (&u)[L::D], float (&geq)[L::Q]) {
  constexpr float S = shift_scale<SK>();
  float usq = u[0] * u[0];
#pragma unroll
  for (int d = 1; d < L::D; ++d) usq = __fmaf_rn(u[d], u[d], usq);
  const float b = -1.5f * usq;
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    float cu = 0.0f;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) cu = cu + u[d];
      if (L::c(l, d) == -1) cu = cu - u[d];
    }
    const float t = 3.0f * cu;
    const float em1 = __fmaf_rn(0.5f * t, t, t + b);
    const float e = 1.0f + em1;
    geq[l] = (S * (float)weight<L>(l)) * __fmaf_rn(drho, e, em1);
  }
}

// ZouHe / Regularized, velocity or pressure, on deviations.  XLB's
// fsum = sum_{opp l missing} 2 f_l + sum_{l, opp l present} f_l equals
// 1 + dW + G/S, G the same sum over g and dW the weights of the directions that
// are missing together with their opposite (0 on a face), so
//   velocity (u = -aux n, u.n = -aux): rho - 1 = (fsum - 1 - u.n) / (1 + u.n),
//   pressure (rho = aux):              u.n = (fsum - 1 - (rho - 1)) / rho,
// then the non-equilibrium bounce-back and the regularisation as in zouhe_like
// (every step linear in g except through rho and u).
template <class L, int SK>
__device__ __forceinline__ void zouhe_like_dev(float (&g)[L::Q], uint32_t miss, float aux, int kind) {
  constexpr float S = shift_scale<SK>();
  constexpr float K = 1.0f / S;
  int nv[L::D];
  normal_of<L>(miss, nv);
  float G = 0.0f, dW = 0.0f;
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    const bool k = (miss >> opp<L>(l)) & 1u;
    const bool m = !k && !((miss >> l) & 1u);
    if (k) G = G + 2.0f * g[l];
    if (m) G = G + g[l];
    if (k && ((miss >> l) & 1u)) dW = dW + (float)weight<L>(l);
  }
  const float fs1 = __fmaf_rn(K, G, dW);  // fsum - 1
  float drho, u[L::D];
  if (kind == BC_ZOUHE_V || kind == BC_REG_V) {
    float unormal = 0.0f;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = (-aux) * (float)nv[d];
#pragma unroll
    for (int d = 0; d < L::D; ++d) unormal = unormal + u[d] * (float)nv[d];
    drho = (fs1 - unormal) / (1.0f + unormal);
  } else {
    drho = aux - 1.0f;
    const float unormal = (fs1 - drho) / aux;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = unormal * (float)nv[d];
  }
  float geq[L::Q];
  equilibrium_dev<L, SK>(drho, u, geq);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    if ((miss >> l) & 1u) g[l] = g[opp<L>(l)] + geq[l] - geq[opp<L>(l)];
  }
  if (kind == BC_REG_V || kind == BC_REG_P) {
    float gneq[L::Q];
#pragma unroll
    for (int l = 0; l < L::Q; ++l) gneq[l] = g[l] - geq[l];
    float pi[L::NT];
    second_moment<L>(gneq, pi);
#pragma unroll
    for (int l = 0; l < L::Q; ++l) {
      float acc = 0.0f;
#pragma unroll
      for (int t = 0; t < L::NT; ++t) {
        if (qi<L>(l, t) != 0.0) acc = acc + (float)qi<L>(l, t) * pi[t];
      }
      g[l] = geq[l] + 4.5f * (float)weight<L>(l) * acc;
    }
  }
}

}  // namespace xlbg
