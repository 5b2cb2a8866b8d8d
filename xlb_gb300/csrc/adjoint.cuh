// Hand-written adjoint of the fused step.
//
// The forward step maps the state f_t to f_{t+1}; per cell y
//   f_{t+1}(y) = F_y(P, O, E, a)
// with P_l = f_t[l](y - c_l) the pulled values (one-cell periodic wrap),
// O = f_t(y) the own-cell values read by HalfwayBounceBack and
// ExtrapolationOutflow (bc_halfway_bounce_back.py:67-85,
// bc_extrapolation_outflow.py:138-195), E_l = f_t[l](y - c_l - n) the
// extrapolation neighbour values, and a the ZouHe / Regularized prescribed value
// (bc_zouhe.py:279-343, bc_regularized.py:134-202).  Given lam_out =
// dL/df_{t+1}, the reverse step forms lam_in = dL/df_t as the sum over cells of
// the transposed local Jacobians:
//   pass 1, every cell: a fluid cell pushes the P part to lam_in[l](y - c_l).
//     For each l the pull is a bijection of the cells, so every lam_in element
//     has exactly one pusher and takes a plain store: the reverse push-stream.
//     A boundary cell stores zeros to its push targets instead.
//   pass 2, the boundary cells (id != 0) only: the full local adjoint, whose P
//     part is added atomically to the zeros of pass 1 and whose O and E parts
//     are added atomically wherever they land; dL/da is added to aux_grad.
//     Additions commute, so pass 2 needs no ordering among its threads.
// Pass 1 thus runs the short fluid adjoint only (few registers, full
// occupancy) and the boundary code runs on the surface cells alone.
// Per cell the local Jacobian is applied in reverse program order:
// collision-step BC, collision (BGK or KBC with the macroscopic and quadratic
// equilibrium operators), streaming-step BC.  Each operator's adjoint below is
// written out by hand from the forward functional it names.
//
// Arithmetic is in the compute type T.  Cells with id 255 are not supported
// (their populations are never rewritten, so f_{t+1} would depend on f_{t-1});
// their threads write zero to their push targets so the output is defined.
#pragma once
#include "step_kernel.cuh"

namespace xlbg {

struct AdjArgs {
  StepArgs s;              // s.f0: forward input state f_t; s.aux: aux plane; s.f1 unused
  const void* lam_out;     // dL/df_{t+1}, compute type, Q planes
  void* lam_in;            // dL/df_t, compute type, Q planes
  const long long* bc_cells;  // pass 2: sorted linear indices of every cell with id != 0
  long long n_bc;
  void* aux_grad;          // pass 2: n_bc values, += dL/da at ZouHe / Regularized cells
};

// ---- equilibrium (quadratic_equilibrium.py:35-60) ----
// feq_l = rho w_l (1 + cu_l (1 + cu_l / 2) - usqr), cu_l = 3 c_l.u, usqr = 1.5 |u|^2.
template <class L, class T>
__device__ __forceinline__ void equilibrium_adj(T rho, const T (&u)[L::D], const T (&feqb)[L::Q], T& rhob,
                                                T (&ub)[L::D]) {
  const T usqr = usqr_of<L>(u);
  T usqrb = T(0);
  rhob = T(0);
#pragma unroll
  for (int d = 0; d < L::D; ++d) ub[d] = T(0);
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    T cu = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) cu = cu + u[d];
      if (L::c(l, d) == -1) cu = cu - u[d];
    }
    cu = cu * T(3);
    const T wl = T(weight<L>(l));
    rhob = rhob + feqb[l] * wl * (T(1) + cu * (T(1) + T(0.5) * cu) - usqr);
    const T t = feqb[l] * rho * wl;
    usqrb = usqrb - t;
    const T cub = T(3) * t * (T(1) + cu);
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) ub[d] = ub[d] + cub;
      if (L::c(l, d) == -1) ub[d] = ub[d] - cub;
    }
  }
#pragma unroll
  for (int d = 0; d < L::D; ++d) ub[d] = ub[d] + T(3) * u[d] * usqrb;
}

// ---- macroscopic (zero_moment.py:22-27, first_moment.py:25-38) ----
// rho = sum f, u_d = m_d / rho with m_d = sum_l c_ld f_l.  Adds into fb.
template <class L, class T>
__device__ __forceinline__ void macroscopic_adj(T rho, const T (&u)[L::D], T rhob, const T (&ub)[L::D],
                                                T (&fb)[L::Q]) {
  const T inv = T(1) / rho;
  T mb[L::D];
  T r = rhob;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    mb[d] = ub[d] * inv;
    r = r - ub[d] * u[d] * inv;
  }
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    T v = r;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) v = v + mb[d];
      if (L::c(l, d) == -1) v = v - mb[d];
    }
    fb[l] = fb[l] + v;
  }
}

// ---- KBC shear part (kbc.py:193-250) without the rho factor ----
template <class L, class T>
__device__ __forceinline__ void kbc_shear(const T (&pi)[L::NT], T (&s)[L::Q]) {
#pragma unroll
  for (int l = 0; l < L::Q; ++l) s[l] = T(0);
  if constexpr (L::Q == 27) {
    const T nxz = pi[0] - pi[5];
    const T nyz = pi[3] - pi[5];
    const T a = (T(2) * nxz - nyz) / T(6);
    const T b = (-nxz + T(2) * nyz) / T(6);
    const T cz = (-nxz - nyz) / T(6);
    const T p1 = pi[1] / T(4), p2 = pi[2] / T(4), p4 = pi[4] / T(4);
    s[9] = a; s[18] = a; s[3] = b; s[6] = b; s[1] = cz; s[2] = cz;
    s[12] = p1; s[24] = p1; s[21] = -p1; s[15] = -p1;
    s[10] = p2; s[20] = p2; s[19] = -p2; s[11] = -p2;
    s[8] = p4; s[4] = p4; s[7] = -p4; s[5] = -p4;
  } else {
    const T n = pi[0] - pi[2];
    s[3] = n; s[6] = n; s[2] = -n; s[1] = -n;
    s[8] = pi[1]; s[4] = -pi[1]; s[5] = -pi[1]; s[7] = pi[1];
  }
}

// transpose of kbc_shear
template <class L, class T>
__device__ __forceinline__ void kbc_shear_adj(const T (&sb)[L::Q], T (&pib)[L::NT]) {
  if constexpr (L::Q == 27) {
    const T ab = sb[9] + sb[18], bb = sb[3] + sb[6], cb = sb[1] + sb[2];
    const T nxzb = (T(2) * ab - bb - cb) / T(6);
    const T nyzb = (-ab + T(2) * bb - cb) / T(6);
    pib[0] = nxzb;
    pib[3] = nyzb;
    pib[5] = -nxzb - nyzb;
    pib[1] = (sb[12] + sb[24] - sb[21] - sb[15]) / T(4);
    pib[2] = (sb[10] + sb[20] - sb[19] - sb[11]) / T(4);
    pib[4] = (sb[8] + sb[4] - sb[7] - sb[5]) / T(4);
  } else {
    const T nb = sb[3] + sb[6] - sb[2] - sb[1];
    pib[0] = nb;
    pib[2] = -nb;
    pib[1] = sb[8] - sb[4] - sb[5] + sb[7];
  }
}

// ---- KBC (kbc.py:192-296), D2Q9 and D3Q27 ----
// fneq = f - feq, ds = kappa rho s(Pi(fneq)) (kappa 1 for D3Q27, 1/4 for D2Q9),
// dh = fneq - ds, sp1 = sum dh ds / feq, sp2 = sum dh^2 / feq,
// gamma = 1/beta - (2 - 1/beta) sp1 / (1e-32 + sp2), fo = f - beta (2 ds + gamma dh).
// Sets fb from fob.
template <class L, class T>
__device__ __forceinline__ void kbc_adj(const T (&f)[L::Q], T rho, const T (&u)[L::D], T omega,
                                        const T (&fob)[L::Q], T (&fb)[L::Q]) {
  constexpr int Q = L::Q;
  const T kap = Q == 27 ? T(1) : T(0.25);
  T feq[Q];
  equilibrium<L>(rho, u, feq);
  T fneq[Q];
#pragma unroll
  for (int l = 0; l < Q; ++l) fneq[l] = f[l] - feq[l];
  T pi[L::NT];
  second_moment<L>(fneq, pi);
  T s[Q];
  kbc_shear<L>(pi, s);
  T ds[Q], dh[Q];
  T sp1 = T(0), sp2 = T(0);
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    ds[l] = s[l] * rho * kap;
    dh[l] = fneq[l] - ds[l];
    const T temp = dh[l] / feq[l];
    sp1 = sp1 + temp * ds[l];
    sp2 = sp2 + temp * dh[l];
  }
  const T beta = T(0.5) * omega;
  const T ib = T(1) / beta;
  const T cc2 = T(2) - ib;
  const T den = T(1e-32) + sp2;
  const T gamma = ib - cc2 * sp1 / den;
  T gb = T(0);
#pragma unroll
  for (int l = 0; l < Q; ++l) gb = gb - beta * fob[l] * dh[l];
  const T sp1b = -cc2 * gb / den;
  const T sp2b = cc2 * sp1 * gb / (den * den);
  // reuse: fneq <- adjoint of fneq, s <- adjoint of ds, feq stays, dh/ds forward
  T feqb[Q];
  T rhob = T(0);
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    fb[l] = fob[l];
    const T ifeq = T(1) / feq[l];
    const T dsb = T(-2) * beta * fob[l] + sp1b * dh[l] * ifeq;
    const T dhb = -beta * gamma * fob[l] + (sp1b * ds[l] + T(2) * sp2b * dh[l]) * ifeq;
    feqb[l] = -(sp1b * dh[l] * ds[l] + sp2b * dh[l] * dh[l]) * ifeq * ifeq;
    const T dsb2 = dsb - dhb;        // dh = fneq - ds
    rhob = rhob + kap * s[l] * dsb2;  // ds = kap rho s
    fneq[l] = dhb;
    s[l] = kap * rho * dsb2;
  }
  T pib[L::NT];
  kbc_shear_adj<L>(s, pib);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    T v = fneq[q];
#pragma unroll
    for (int t = 0; t < L::NT; ++t) {
      if (cc<L>(q, t) == 1) v = v + pib[t];
      if (cc<L>(q, t) == -1) v = v - pib[t];
    }
    fb[q] = fb[q] + v;      // fneq = f - feq
    feqb[q] = feqb[q] - v;
  }
  T rhob2, ub[L::D];
  equilibrium_adj<L>(rho, u, feqb, rhob2, ub);
  macroscopic_adj<L>(rho, u, rhob + rhob2, ub, fb);
}

// Collision adjoint: BGK (bgk.py:30-34; also for the pair form, which has the
// same equations) or KBC.  Sets fb from fob; f are the post-streaming values.
template <class L, class T, bool KBC>
__device__ __forceinline__ void collide_adj(const T (&f)[L::Q], T omega, const T (&fob)[L::Q], T (&fb)[L::Q]) {
  T rho, u[L::D];
  macroscopic<L>(f, rho, u);
  if constexpr (KBC) {
    kbc_adj<L>(f, rho, u, omega, fob, fb);
  } else {
    // fo = f - omega (f - feq)
    T feqb[L::Q];
#pragma unroll
    for (int l = 0; l < L::Q; ++l) {
      fb[l] = (T(1) - omega) * fob[l];
      feqb[l] = omega * fob[l];
    }
    T rhob, ub[L::D];
    equilibrium_adj<L>(rho, u, feqb, rhob, ub);
    macroscopic_adj<L>(rho, u, rhob, ub, fb);
  }
}

// ---- ZouHe / Regularized (bc_zouhe.py:279-343, bc_regularized.py:134-202,
// helper_functions_bc.py:236-297), forward as zouhe_like in physics.cuh ----
// In: P the pulled values, gb the adjoint of the BC output.  Out: gb holds the
// adjoint of P, auxb the derivative with respect to the prescribed value.
template <class L, class T>
__device__ __forceinline__ void zouhe_adj(const T (&P)[L::Q], uint32_t miss, T aux, int kind, T (&gb)[L::Q],
                                          T& auxb) {
  constexpr int Q = L::Q;
  int nv[L::D];
  normal_of<L>(miss, nv);
  T known = T(0), middle = T(0);
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    const bool k = (miss >> opp<L>(l)) & 1u;
    const bool m = !k && !((miss >> l) & 1u);
    if (k) known = known + T(2) * P[l];
    if (m) middle = middle + P[l];
  }
  const T fsum = known + middle;
  const bool vel = kind == BC_ZOUHE_V || kind == BC_REG_V;
  T rho, u[L::D], unormal;
  if (vel) {
    unormal = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = (-aux) * T(nv[d]);
#pragma unroll
    for (int d = 0; d < L::D; ++d) unormal = unormal + u[d] * T(nv[d]);
    rho = fsum / (T(1) + unormal);
  } else {
    rho = aux;
    unormal = T(-1) + fsum / rho;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d] = unormal * T(nv[d]);
  }
  T feqb[Q];
#pragma unroll
  for (int l = 0; l < Q; ++l) feqb[l] = T(0);
  if (kind == BC_REG_V || kind == BC_REG_P) {
    // out_l = feq_l + 4.5 w_l sum_t qi_lt Pi_t(g - feq)
    T pib[L::NT];
#pragma unroll
    for (int t = 0; t < L::NT; ++t) {
      T acc = T(0);
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        if (qi<L>(l, t) != 0.0) acc = acc + T(qi<L>(l, t)) * T(4.5) * T(weight<L>(l)) * gb[l];
      }
      pib[t] = acc;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T v = T(0);
#pragma unroll
      for (int t = 0; t < L::NT; ++t) {
        if (cc<L>(q, t) == 1) v = v + pib[t];
        if (cc<L>(q, t) == -1) v = v - pib[t];
      }
      feqb[q] = gb[q] - v;
      gb[q] = v;
    }
  }
  // non-equilibrium bounce-back, in place in ascending l in the forward
  // (helper_functions_bc.py:263-272), so reversed in descending l
#pragma unroll
  for (int l = Q - 1; l >= 0; --l) {
    if (opp<L>(l) != l && ((miss >> l) & 1u)) {
      const T v = gb[l];
      gb[opp<L>(l)] = gb[opp<L>(l)] + v;
      feqb[l] = feqb[l] + v;
      feqb[opp<L>(l)] = feqb[opp<L>(l)] - v;
      gb[l] = T(0);
    }
  }
  T rhob, ub[L::D];
  equilibrium_adj<L>(rho, u, feqb, rhob, ub);
  T fsumb;
  if (vel) {
    const T den = T(1) + unormal;
    fsumb = rhob / den;
    const T unb = -rhob * rho / den;
    T s = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) s = s + (ub[d] + unb * T(nv[d])) * T(nv[d]);
    auxb = -s;
  } else {
    T unb = T(0);
#pragma unroll
    for (int d = 0; d < L::D; ++d) unb = unb + ub[d] * T(nv[d]);
    fsumb = unb / rho;
    auxb = rhob - unb * fsum / (rho * rho);
  }
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    const bool k = (miss >> opp<L>(l)) & 1u;
    const bool m = !k && !((miss >> l) & 1u);
    if (k) gb[l] = gb[l] + T(2) * fsumb;
    if (m) gb[l] = gb[l] + fsumb;
  }
}

// Reverse of one boundary cell.  g holds lam_out at the cell on entry and the
// adjoint of the pulled values P on return (the caller pushes it); the
// own-cell, extrapolation-neighbour and aux terms are added here, atomically.
template <class L, int SK, class T, bool KBC>
__device__ __forceinline__ void cell_adjoint(const AdjArgs& A, int i0, int i1, int i2, long long cell, uint8_t id,
                                             const T (&P)[L::Q], T (&g)[L::Q], long long list_index) {
  const StepArgs& a = A.s;
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;
  T* __restrict__ lam_in = static_cast<T*>(A.lam_in);
  const long long N = a.ncell;
  int kind = 0;
  if (id != 0) kind = (int)(a.bc_code[id] & 0xffu);
  if (kind == BC_EQUILIBRIUM) {  // f_post_stream = feq(rho_bc, u_bc): no dependence on f_t
#pragma unroll
    for (int l = 0; l < Q; ++l) g[l] = T(0);
    return;
  }
  const bool own_kind = kind == BC_HALFWAY || kind == BC_EXTRAP;
  const bool zh_kind = kind >= BC_ZOUHE_V && kind <= BC_REG_P;
  const uint32_t miss = (own_kind || zh_kind) ? __ldg(a.miss + cell) : 0u;

  // forward: post-streaming values
  T fps[Q];
#pragma unroll
  for (int l = 0; l < Q; ++l) fps[l] = P[l];
  T aux = T(0);
  if (own_kind) {
#pragma unroll
    for (int l = 0; l < Q; ++l)
      if ((miss >> l) & 1u) fps[l] = St::dec(ldg_bits(at0<Bits>(a, opp<L>(l), cell)), T(weight<L>(opp<L>(l))));
  } else if (zh_kind) {
    aux = St::dec_raw(static_cast<const Bits*>(a.aux)[cell]);
    zouhe_like<L>(fps, miss, aux, kind);
  }

  // reverse: collision-step BC and collision -> fb, the adjoint of fps
  T fb[Q];
  if (kind == BC_FULLWAY) {
    // f_out[l] = f_post_stream[opp l] (bc_fullway_bounce_back.py:59-72)
#pragma unroll
    for (int l = 0; l < Q; ++l) fb[opp<L>(l)] = g[l];
  } else if (kind == BC_EXTRAP) {
    // f_out[opp l] = (1 - cs) f_post_stream[l] + cs E_l for missing l
    // (bc_extrapolation_outflow.py:390-415); those slots drop the collision output
    int nv[L::D];
    normal_of<L>(miss, nv);
    const T cs = T(a.extrap_cs);
    const int m0 = L::D == 3 ? nv[0] : 0;
    const int m1 = L::D == 3 ? nv[1] : nv[0];
    const int m2 = L::D == 3 ? nv[2] : nv[1];
    T ex[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      ex[l] = T(0);
      if ((miss >> l) & 1u) {
        const T v = g[opp<L>(l)];
        ex[l] = (T(1) - cs) * v;
        {
          const int s0 = wrap_any(i0 - (axis_c<L>(l, 0) + m0), a.n0);
          const int s1 = wrap_any(i1 - (axis_c<L>(l, 1) + m1), a.n1);
          const int s2 = wrap_any(i2 - (axis_c<L>(l, 2) + m2), a.n2);
          const long long src = ((long long)s0 * a.n1 + s1) * a.n2 + s2;
          atomicAdd(lam_in + (long long)l * N + src, cs * v);
        }
        g[opp<L>(l)] = T(0);
      }
    }
    collide_adj<L, T, KBC>(fps, omega_of<T>(a), g, fb);
#pragma unroll
    for (int l = 0; l < Q; ++l) fb[l] = fb[l] + ex[l];
  } else {
    collide_adj<L, T, KBC>(fps, omega_of<T>(a), g, fb);
  }

  // reverse: streaming-step BC -> g, the adjoint of P
  if (own_kind) {
    // f_post_stream[l] = f_pre[opp l] for missing l
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      if ((miss >> l) & 1u) {
        atomicAdd(lam_in + (long long)opp<L>(l) * N + cell, fb[l]);
        g[l] = T(0);
      } else {
        g[l] = fb[l];
      }
    }
  } else if (zh_kind) {
    T auxb;
    zouhe_adj<L>(P, miss, aux, kind, fb, auxb);
#pragma unroll
    for (int l = 0; l < Q; ++l) g[l] = fb[l];
    {
      T* ag = static_cast<T*>(A.aux_grad);
      ag[list_index] = ag[list_index] + auxb;
    }
  } else {
#pragma unroll
    for (int l = 0; l < Q; ++l) g[l] = fb[l];
  }
}

// Pull source of direction l of cell (i0, i1, i2), with the one-cell wrap; also
// the push target of the reverse stream.
template <class L>
__device__ __forceinline__ long long pull_source(const RowOffsets& rows, const int (&z)[3], int l) {
  return rows.of<L>(l) + z[axis_c<L>(l, 2) + 1];
}

// Pass 1: every cell, one thread per cell; grid as step_kernel.  Fluid cells
// run the collision adjoint and push; boundary cells zero their push targets.
// Resident blocks asked of the register allocator for pass 1: the forward
// kernel's choice for BGK; KBC's adjoint keeps the allocator's choice (its
// per-cell state does not fit the BGK budget).
template <class L, class T, bool KBC>
constexpr int adjoint_min_blocks() {
  return KBC ? 1 : march_min_blocks<L, T>();
}

template <class L, int SK, class T, bool KBC>
__global__ void __launch_bounds__(kStepBlock, adjoint_min_blocks<L, T, KBC>()) adjoint_push_kernel(const AdjArgs A) {
  const StepArgs& a = A.s;
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;
  const int n1 = a.n1, n2 = a.n2;
  const int row = blockIdx.x;
  const int i0 = row / n1;
  const int i1 = row - i0 * n1;
  const int i2 = blockIdx.y * blockDim.x + threadIdx.x;
  if (i2 >= n2) return;
  const long long cell = (long long)row * n2 + i2;
  const long long N = a.ncell;
  const RowOffsets rows(i0, i1, a.n0, n1, n2);
  const int z[3] = {i2 == n2 - 1 ? 0 : i2 + 1, i2, i2 == 0 ? n2 - 1 : i2 - 1};
  const T* __restrict__ lam_out = static_cast<const T*>(A.lam_out);
  T* __restrict__ lam_in = static_cast<T*>(A.lam_in);
  if (a.bc_mask[cell] != 0) {
#pragma unroll
    for (int l = 0; l < Q; ++l) lam_in[(long long)l * N + pull_source<L>(rows, z, l)] = T(0);
    return;
  }
  T P[Q], g[Q], fb[Q];
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    P[l] = St::dec(ldg_bits(at0<Bits>(a, l, pull_source<L>(rows, z, l))), T(weight<L>(l)));
    g[l] = lam_out[(long long)l * N + cell];
  }
  collide_adj<L, T, KBC>(P, omega_of<T>(a), g, fb);
#pragma unroll
  for (int l = 0; l < Q; ++l) lam_in[(long long)l * N + pull_source<L>(rows, z, l)] = fb[l];
}

// Pass 2: every boundary cell (id != 0), one thread per cell; all writes are
// atomic additions.
template <class L, int SK, class T, bool KBC>
__global__ void __launch_bounds__(kStepBlock) adjoint_bc_kernel(const AdjArgs A) {
  const StepArgs& a = A.s;
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_bc) return;
  const long long cell = A.bc_cells[i];
  const int n1 = a.n1, n2 = a.n2;
  const long long plane = (long long)n1 * n2;
  const int i0 = (int)(cell / plane);
  const long long rem = cell - (long long)i0 * plane;
  const int i1 = (int)(rem / n2);
  const int i2 = (int)(rem - (long long)i1 * n2);
  const uint8_t id = a.bc_mask[cell];
  if (id == 0 || id == 255) return;
  const long long N = a.ncell;
  const RowOffsets rows(i0, i1, a.n0, n1, n2);
  const int z[3] = {i2 == n2 - 1 ? 0 : i2 + 1, i2, i2 == 0 ? n2 - 1 : i2 - 1};
  const T* __restrict__ lam_out = static_cast<const T*>(A.lam_out);
  T* __restrict__ lam_in = static_cast<T*>(A.lam_in);
  T P[Q], g[Q];
#pragma unroll
  for (int l = 0; l < Q; ++l) {
    P[l] = St::dec(ldg_bits(at0<Bits>(a, l, pull_source<L>(rows, z, l))), T(weight<L>(l)));
    g[l] = lam_out[(long long)l * N + cell];
  }
  cell_adjoint<L, SK, T, KBC>(A, i0, i1, i2, cell, id, P, g, i);
#pragma unroll
  for (int l = 0; l < Q; ++l) atomicAdd(lam_in + (long long)l * N + pull_source<L>(rows, z, l), g[l]);
}

// Launch of both passes for one lattice; returns 0, -1 (unsupported pair) or the CUDA error.
template <int LAT>
int launch_adjoint_t(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s) {
  using L = Lattice<LAT>;
  const StepArgs& a = A.s;
  const dim3 grid((unsigned)(a.n0 * a.n1), (unsigned)((a.n2 + kStepBlock - 1) / kStepBlock));
  const unsigned bgrid = (unsigned)((A.n_bc + kStepBlock - 1) / kStepBlock);
#define XLBG_ALAUNCH(SKV, TV, K)                                                    \
  do {                                                                              \
    adjoint_push_kernel<L, SKV, TV, K><<<grid, kStepBlock, 0, s>>>(A);              \
    if (A.n_bc > 0) adjoint_bc_kernel<L, SKV, TV, K><<<bgrid, kStepBlock, 0, s>>>(A); \
  } while (0)
  if (LAT == 1 && kbc) return -1;
  if (compute == 1 && sk == SK_F64) {
    if (kbc) XLBG_ALAUNCH(SK_F64, double, (LAT != 1)); else XLBG_ALAUNCH(SK_F64, double, false);
  } else if (compute == 1 && sk == SK_F32) {
    if (kbc) XLBG_ALAUNCH(SK_F32, double, (LAT != 1)); else XLBG_ALAUNCH(SK_F32, double, false);
  } else if (compute == 0 && sk == SK_F32) {
    if (kbc) XLBG_ALAUNCH(SK_F32, float, (LAT != 1)); else XLBG_ALAUNCH(SK_F32, float, false);
  } else {
    return -1;
  }
#undef XLBG_ALAUNCH
  return (int)cudaGetLastError();
}

int launch_adjoint_d2q9(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s);
int launch_adjoint_d3q19(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s);
int launch_adjoint_d3q27(const AdjArgs& A, int sk, int compute, bool kbc, cudaStream_t s);

}  // namespace xlbg
