// Two-cell collision for BGK on the stored deviations of the shifted 16-bit
// stores (collision code 3, and code 4 with stochastic rounding), used by the
// segmented step kernel (step_tma_seg.cuh).
//
// A consumer thread owns two adjacent cells of a row and carries every value of
// the collision as a pair of floats in one 64-bit register, operated on by
// Blackwell's packed FP32 instructions (fma/add/sub/mul.rn.f32x2).  Each lane of
// a packed instruction is the scalar instruction of bgk_shifted, in the same
// order with the same rounding, so the results are bit-identical to the one-cell
// kernels and the oracle.  Unlike scalar .rn arithmetic, a packed mul.rn.f32x2
// whose only use is a packed add can be contracted by ptxas into a packed FMA
// (measured: a direction-paired equilibrium written that way differed from the
// scalar one in 0.4 % of values), so every fused step here is an explicit fma2
// and no single-use mul2 feeds an add2 / sub2; the parity tests check the bits
// at every size.  The two cells'
// values of a direction convert with one cvt.rn.{f16x2,bf16x2} and store as one
// 32-bit word (the pair is 4-byte aligned: rows hold a multiple of 8 cells).
// With stochastic rounding (code 4) the conversion is cvt.rs with each half
// given the 16 random bits the one-cell store gives that (cell, direction), so
// results stay identical too.
#pragma once
#include <type_traits>

#include "step_kernel.cuh"

namespace xlbg {

using f2 = unsigned long long;  // two floats: cell 2j in the low half, 2j + 1 in the high half

__device__ __forceinline__ f2 pk2(float lo, float hi) {
  f2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ float lo2(f2 a) {
  float l, h;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(l), "=f"(h) : "l"(a));
  return l;
}
__device__ __forceinline__ float hi2(f2 a) {
  float l, h;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(l), "=f"(h) : "l"(a));
  return h;
}
__device__ __forceinline__ f2 dup2(float x) { return pk2(x, x); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Pair moments of bgk_shifted (pair_moments' order): G += g_l + g_o, J_d +-= g_l - g_o.
template <class L, int P>
__device__ __forceinline__ void pair_moments2(const f2 (&g)[L::Q], f2& G, f2 (&J)[L::D]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    const f2 sig = add2(g[l], g[o]);
    const f2 dif = sub2(g[l], g[o]);
    G = add2(G, sig);
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      // J starts at 0: 0 + x and 0 - x are x and -x exactly (0 - x of x = 0 is +0,
      // as the scalar code gives)
      if (L::c(l, d) == 1) J[d] = add2(J[d], dif);
      if (L::c(l, d) == -1) J[d] = sub2(J[d], dif);
    }
    pair_moments2<L, P + 1>(g, G, J);
  }
}

// The pair update of bgk_shifted for pair P.  t = c_l . v is sigma * s with s
// formed from v by adds / subtracts in the scalar order; RN commutes with the
// sign, so fma(A, t, R) = fma(sigma A, s, R) and fma(Arh t, t, C) = fma(Arh s, s, C).
template <class L, int P>
__device__ __forceinline__ void shifted_pair_update2(f2 (&g)[L::Q], const f2 (&v)[L::D], const f2 (&Ar)[4],
                                                     const f2 (&nAr)[4], const f2 (&Arh)[4], const f2 (&C)[4],
                                                     f2 omf) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    constexpr int k = norm1<L>(l);
    // s = |first nonzero component sign| * t: the scalar code forms t = x_1 (+ x_2 ...) with
    // x_d = +-v_d; with sigma the sign of the first component, s = v_a (+-) v_b ...
    constexpr int d0 = L::c(l, 0) != 0 ? 0 : (L::c(l, 1) != 0 ? 1 : 2);
    constexpr int sigma = L::c(l, d0);
    f2 s = v[d0];
#pragma unroll
    for (int d = d0 + 1; d < L::D; ++d) {
      if (L::c(l, d) != 0) s = (L::c(l, d) == sigma) ? add2(s, v[d]) : sub2(s, v[d]);
    }
    const f2 R = fma2(mul2(Arh[k], s), s, C[k]);
    const f2 Al = sigma > 0 ? Ar[k] : nAr[k];
    const f2 Ao = sigma > 0 ? nAr[k] : Ar[k];
    g[l] = fma2(omf, g[l], fma2(Al, s, R));
    g[o] = fma2(omf, g[o], fma2(Ao, s, R));
    shifted_pair_update2<L, P + 1>(g, v, Ar, nAr, Arh, C, omf);
  }
}

// bgk_shifted on two cells at once, in place (g holds the outputs on return).
template <class L, int SK>
__device__ __forceinline__ void bgk_shifted2(f2 (&g)[L::Q], float omega) {
  constexpr float S = shift_scale<SK>();
  constexpr float K = 1.0f / S;
  f2 G = g[0];
  f2 J[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) J[d] = dup2(0.0f);
  pair_moments2<L, 0>(g, G, J);
  const f2 K2 = dup2(K);
  const f2 rho = fma2(K2, G, dup2(1.0f));
  const f2 inv = pk2(__frcp_rn(lo2(rho)), __frcp_rn(hi2(rho)));
  const f2 k3 = mul2(dup2(3.0f), mul2(K2, inv));
  f2 v[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) v[d] = mul2(J[d], k3);
  f2 vsq = mul2(v[0], v[0]);
#pragma unroll
  for (int d = 1; d < L::D; ++d) vsq = fma2(v[d], v[d], vsq);
  const f2 bm1 = mul2(dup2(-1.0f / 6.0f), vsq);
  const f2 base = add2(dup2(1.0f), bm1);
  const f2 r = fma2(mul2(K2, G), base, bm1);
  const f2 omf = dup2(1.0f - omega);
  constexpr double Sw[4] = {(double)S * class_weight<L>(0), (double)S * class_weight<L>(1),
                            (double)S * class_weight<L>(2), (double)S * class_weight<L>(3)};
  constexpr float Whi[4] = {(float)Sw[0], (float)Sw[1], (float)Sw[2], (float)Sw[3]};
  constexpr float Wlo[4] = {(float)(Sw[0] - (double)Whi[0]), (float)(Sw[1] - (double)Whi[1]),
                            (float)(Sw[2] - (double)Whi[2]), (float)(Sw[3] - (double)Whi[3])};
  f2 Ar[4], nAr[4], Arh[4], C[4];
#pragma unroll
  for (int k = 0; k <= L::D; ++k) {
    const float Ahi = omega * Whi[k];
    const float Alo = __fmaf_rn(omega, Whi[k], -Ahi) + omega * Wlo[k];
    const f2 AH = dup2(Ahi), AL = dup2(Alo);
    Ar[k] = fma2(AH, rho, mul2(AL, rho));
    nAr[k] = sub2(dup2(0.0f), Ar[k]);  // -Ar exactly (Ar > 0)
    Arh[k] = mul2(dup2(0.5f), Ar[k]);
    C[k] = fma2(AH, r, mul2(AL, r));
  }
  g[0] = fma2(omf, g[0], C[0]);
  shifted_pair_update2<L, 0>(g, v, Ar, nAr, Arh, C, omf);
}

template <int SK>
__device__ __forceinline__ uint32_t pack_rn2(f2 x) {
  uint32_t d;
  if constexpr (SK == SK_F16S)
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi2(x)), "f"(lo2(x)));
  else
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi2(x)), "f"(lo2(x)));
  return d;
}

// Mass of the two cells of a stored 32-bit pair word p of direction l, decoded
// as the one-cell store decodes it and summed in FP32 in direction order (the
// diagnostics step's per-cell mass).
template <class L, int SK>
__device__ __forceinline__ void stored_mass2(uint32_t p, int l, float& m0, float& m1) {
  using St = Store<SK, float>;
  using Bits = typename St::Bits;
  const float v0 = St::dec((Bits)(p & 0xffffu), float(weight<L>(l)));
  const float v1 = St::dec((Bits)(p >> 16), float(weight<L>(l)));
  m0 = l == 0 ? v0 : m0 + v0;
  m1 = l == 0 ? v1 : m1 + v1;
}

// Collision and store of two neighbouring cells of a row (plane i0, row y,
// contiguous-axis index z and z + 1, flat index cell and cell + 1; cell even)
// from their pulled deviations g (low half: cell, high half: cell + 1), as the
// segmented kernel does it: warps whose 64 cells are all fluid take the packed
// collision and one 32-bit store per direction; any other warp runs
// cell_update on its two cells one after the other (boundary cells, skip cells,
// row ends).  DIAG (the diagnostics step) adds each cell's stored mass to dm
// and, through cell_update, the force on the input to df.
template <class L, int SK, int COLL, bool FULLBC, bool WIDE, bool DIAG = false>
__device__ __forceinline__ void pair_finish(const StepArgs& a, f2 (&g)[L::Q], uint16_t ids, int i0, int y, int z,
                                            unsigned cell, double& dm, double (&df)[3]) {
  using T = float;
  using Idx = typename std::conditional<WIDE, long long, unsigned>::type;
  using Bits = typename Store<SK, T>::Bits;
  constexpr int Q = L::Q;
  const size_t plane = (size_t)a.ncell;
  if (__all_sync(0xffffffffu, ids == 0)) {
    bgk_shifted2<L, SK>(g, omega_of<T>(a));
    float m0 = 0.0f, m1 = 0.0f;
    if constexpr (COLL == 4) {
      // the one-cell store rounds (cell c, direction l) with the low (l even) or
      // high (l odd) 16 bits of sr_bits(sr_seed(c, t), l / 2): assemble those
      // of cells c (low half) and c + 1 (high half) per direction
      const uint32_t s0 = sr_seed(cell, a.timestep), s1 = sr_seed(cell + 1u, a.timestep);
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        const uint32_t w0 = sr_bits(s0, l / 2), w1 = sr_bits(s1, l / 2);
        const uint32_t rb = (l & 1) ? __byte_perm(w0, w1, 0x7632) : __byte_perm(w0, w1, 0x5410);
        uint32_t* __restrict__ dst = reinterpret_cast<uint32_t*>(static_cast<Bits*>(a.f1) + (size_t)l * plane + cell);
        const uint32_t p = sr_pack<SK>(lo2(g[l]), hi2(g[l]), rb);
        *dst = p;
        if constexpr (DIAG) stored_mass2<L, SK>(p, l, m0, m1);
      }
    } else {
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        uint32_t* __restrict__ dst = reinterpret_cast<uint32_t*>(static_cast<Bits*>(a.f1) + (size_t)l * plane + cell);
        const uint32_t p = pack_rn2<SK>(g[l]);
        *dst = p;
        if constexpr (DIAG) stored_mass2<L, SK>(p, l, m0, m1);
      }
    }
    if constexpr (DIAG) {
      dm += (double)m0;
      dm += (double)m1;
    }
  } else {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint8_t id = (uint8_t)(h == 0 ? (ids & 0xffu) : (ids >> 8));
      if (id != 255) {
        T f[Q];
#pragma unroll
        for (int l = 0; l < Q; ++l) f[l] = h == 0 ? lo2(g[l]) : hi2(g[l]);
        if constexpr (DIAG) {
          double dmc = 0.0, dfc[3] = {0.0, 0.0, 0.0};
          cell_update<L, SK, T, COLL, FULLBC, true>(a, i0, y, z + h, (Idx)(cell + (unsigned)h), id, f, dmc, dfc);
          dm += dmc;
          df[0] += dfc[0];
          df[1] += dfc[1];
          df[2] += dfc[2];
        } else {
          cell_update<L, SK, T, COLL, FULLBC, false>(a, i0, y, z + h, (Idx)(cell + (unsigned)h), id, f, dm, df);
        }
      }
    }
  }
}

}  // namespace xlbg
