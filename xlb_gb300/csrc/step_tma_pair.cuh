// TMA-staged step with two cells per consumer thread, for BGK on the stored
// deviations of the shifted 16-bit stores (collision code 3, and code 4 with
// stochastic rounding).
//
// The one-cell consumer of step_kernel_tma spends about 440 instructions a cell
// (issue-bound at ~75 % of the 77 B/cell roof).  Here thread j owns cells 2j and
// 2j + 1 of each staged row and carries every value of the collision as a pair
// of floats in one 64-bit register, operated on by Blackwell's packed FP32
// instructions (fma/add/sub/mul.rn.f32x2).  Each lane of a packed instruction is
// the scalar instruction of bgk_shifted, in the same order with the same
// rounding (explicit .rn: no contraction), so the results are bit-identical to
// the one-cell kernel and the oracle.  The two cells' values of a direction
// convert with one cvt.rn.{f16x2,bf16x2} and store as one 32-bit word (the pair
// is 4-byte aligned: rows hold a multiple of 8 cells).  With stochastic rounding
// (code 4) the conversion is cvt.rs with each half given the 16 random bits the
// one-cell store gives that (cell, direction), so results stay identical too.
//
// Warps whose 64 cells are all fluid take the packed path; any other warp runs
// cell_update on its two cells one after the other.  The ring, the producer warp
// and the bounded waits are step_kernel_tma's.
#pragma once
#include "step_tma.cuh"

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

// Consumers: CT2 = PITCH / 2 threads (thread j owns cells 2j, 2j + 1) plus the
// producer warp.  Launch bounds: two CTAs a SM for PITCH <= 512.
template <int PITCH>
__host__ __device__ constexpr int tma2_consumers() {
  return PITCH / 2;
}
template <int PITCH>
__host__ __device__ constexpr int tma2_min_blocks() {
  return PITCH <= 256 ? 4 : (PITCH == 512 ? 2 : 1);
}

template <class L, int SK, int COLL, bool FULLBC, int PITCH, bool WIDE>
__global__ void __launch_bounds__(tma2_consumers<PITCH>() + 32, tma2_min_blocks<PITCH>())
    step_kernel_tma_pair(const __grid_constant__ CUtensorMap map, const StepArgs a, int rows, int box, int* err) {
  using T = float;
  using Idx = typename std::conditional<WIDE, long long, unsigned>::type;
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  static_assert(sizeof(Bits) == 2, "16-bit stores");
  static_assert(COLL == 3 || COLL == 4, "BGK on deviations");
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned ROW = PITCH * 2;
  constexpr unsigned STAGE = Q * ROW;
  constexpr int CT = tma2_consumers<PITCH>();
  constexpr unsigned CONSUMER_WARPS = CT / 32;
  extern __shared__ __align__(1024) unsigned char smem[];
  const unsigned base = smem_addr(smem);
  const unsigned full = base + S * STAGE;
  const unsigned empty = full + 8 * S;
  const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
  const int i0 = blockIdx.x;
  const int r0 = blockIdx.y * rows;
  const int nr = min(rows, n1 - r0);
  const int tid = threadIdx.x;
  if (base % 128 != 0) {
    if (tid == 0) atomicAdd(err, 1);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full + 8 * s, 1);
      mbar_init(empty + 8 * s, CONSUMER_WARPS);
    }
    fence_barrier_init();
  }
  __syncthreads();

  if (tid >= CT) {
    tma_produce<L, 2, PITCH>(map, base, full, empty, tid - CT, i0, r0, nr, n0, n1, n2, box, err);
    return;
  }

  // ---- consumers: cells c0 = 2 tid and c1 = c0 + 1 of every row ----
  const int lane = tid & 31;
  const int c0 = 2 * tid;
  const bool active = c0 < n2;  // n2 is even: both cells or neither
  // staged-row byte offsets of the sources of c0 and c1 for c2 = -1, 0, +1
  const unsigned za[3] = {(unsigned)(c0 + 1) * 2, (unsigned)c0 * 2, (unsigned)(c0 == 0 ? n2 - 1 : c0 - 1) * 2};
  const unsigned zc[3] = {(unsigned)(c0 + 1 == n2 - 1 ? 0 : c0 + 2) * 2, (unsigned)(c0 + 1) * 2, (unsigned)c0 * 2};
  double dm = 0.0, df[3] = {0.0, 0.0, 0.0};
  const unsigned row0 = ((unsigned)i0 * (unsigned)n1 + (unsigned)r0) * (unsigned)n2 + (unsigned)c0;
  uint16_t ids_next =
      (active && nr > 0) ? *reinterpret_cast<const uint16_t*>(a.bc_mask + row0) : (uint16_t)0xffff;
  const size_t plane = (size_t)a.ncell;
  for (int k = 0; k < nr; ++k) {
    const unsigned s = (unsigned)(k % S);
    const int y = r0 + k;
    const unsigned cell = row0 + (unsigned)k * (unsigned)n2;
    const uint16_t ids = ids_next;
    if (k + 1 < nr)
      ids_next = active ? *reinterpret_cast<const uint16_t*>(a.bc_mask + cell + (unsigned)n2) : (uint16_t)0xffff;
    const bool ok = mbar_wait(full + 8 * s, (unsigned)((k / S) & 1), kTmaWaitNs);
    if (__any_sync(0xffffffffu, !ok)) {
      if (lane == 0) atomicAdd(err, 1);
      return;
    }
    f2 g[Q];
    if (active) {
      const unsigned char* st = smem + s * STAGE;
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        const int cz = axis_c<L>(l, 2);
        float ga, gb;
        if (cz == 0) {  // both sources in one aligned 32-bit word
          const uint32_t w = *reinterpret_cast<const uint32_t*>(st + l * ROW + (unsigned)c0 * 2);
          ga = St::dev((Bits)(w & 0xffffu), 0.0f);
          gb = St::dev((Bits)(w >> 16), 0.0f);
        } else {
          ga = St::dev(*reinterpret_cast<const Bits*>(st + l * ROW + za[cz + 1]), 0.0f);
          gb = St::dev(*reinterpret_cast<const Bits*>(st + l * ROW + zc[cz + 1]), 0.0f);
        }
        g[l] = pk2(ga, gb);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + 8 * s);
    if (__all_sync(0xffffffffu, ids == 0)) {
      // 64 fluid cells: the packed collision, one 32-bit store per direction
      bgk_shifted2<L, SK>(g, omega_of<T>(a));
      if constexpr (COLL == 4) {
        // the one-cell store rounds (cell c, direction l) with the low (l even) or
        // high (l odd) 16 bits of sr_bits(sr_seed(c, t), l / 2): assemble those
        // of cells c0 (low half) and c0 + 1 (high half) per direction
        const uint32_t s0 = sr_seed(cell, a.timestep), s1 = sr_seed(cell + 1u, a.timestep);
#pragma unroll
        for (int l = 0; l < Q; ++l) {
          const uint32_t w0 = sr_bits(s0, l / 2), w1 = sr_bits(s1, l / 2);
          const uint32_t rb = (l & 1) ? __byte_perm(w0, w1, 0x7632) : __byte_perm(w0, w1, 0x5410);
          uint32_t* __restrict__ dst =
              reinterpret_cast<uint32_t*>(static_cast<Bits*>(a.f1) + (size_t)l * plane + cell);
          *dst = sr_pack<SK>(lo2(g[l]), hi2(g[l]), rb);
        }
      } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) {
          uint32_t* __restrict__ dst =
              reinterpret_cast<uint32_t*>(static_cast<Bits*>(a.f1) + (size_t)l * plane + cell);
          *dst = pack_rn2<SK>(g[l]);
        }
      }
    } else {
      // cell by cell through cell_update (boundary cells, skip cells, row ends)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint8_t id = (uint8_t)(h == 0 ? (ids & 0xffu) : (ids >> 8));
        if (id != 255) {
          T f[Q];
#pragma unroll
          for (int l = 0; l < Q; ++l) f[l] = h == 0 ? lo2(g[l]) : hi2(g[l]);
          cell_update<L, SK, T, COLL, FULLBC, false>(a, i0, y, c0 + h, (Idx)(cell + (unsigned)h), id, f, dm, df);
        }
      }
    }
  }
}

template <class L, int SK, int COLL, bool FULLBC, int PITCH, bool WIDE>
int launch_tma_pair_kernel(const CUtensorMap& map, const StepArgs& a, int rows, int box, int* err, cudaStream_t s) {
  const unsigned smem = tma_smem_bytes<L, 2, PITCH>();
  static const bool attr = cudaFuncSetAttribute(step_kernel_tma_pair<L, SK, COLL, FULLBC, PITCH, WIDE>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
  if (!attr) return (int)cudaErrorInvalidValue;
  const dim3 grid((unsigned)a.n0, (unsigned)((a.n1 + rows - 1) / rows));
  step_kernel_tma_pair<L, SK, COLL, FULLBC, PITCH, WIDE>
      <<<grid, tma2_consumers<PITCH>() + 32, smem, s>>>(map, a, rows, box, err);
  return (int)cudaGetLastError();
}

template <class L, int SK, int COLL, int PITCH>
int launch_tma_pair_pitch(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                          cudaStream_t s) {
  if (a.wide)
    return fullbc ? launch_tma_pair_kernel<L, SK, COLL, true, PITCH, true>(map, a, rows, box, err, s)
                  : launch_tma_pair_kernel<L, SK, COLL, false, PITCH, true>(map, a, rows, box, err, s);
  return fullbc ? launch_tma_pair_kernel<L, SK, COLL, true, PITCH, false>(map, a, rows, box, err, s)
                : launch_tma_pair_kernel<L, SK, COLL, false, PITCH, false>(map, a, rows, box, err, s);
}

// Shifted 16-bit stores with collision code 3 or 4 on the two-cell kernel;
// staged rows of 256, 512 or 1024 cells (n2 <= 992, so up to 496 consumers).
// The host checks that bc_mask is 2-byte and f1 4-byte aligned (ids load in
// pairs, outputs store in pairs).
template <int LAT, int SK, int COLL>
int launch_tma_pair_t(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                      cudaStream_t s) {
  using L = Lattice<LAT>;
  if (a.n2 <= 256) return launch_tma_pair_pitch<L, SK, COLL, 256>(map, a, fullbc, rows, box, err, s);
  if (a.n2 <= 512) return launch_tma_pair_pitch<L, SK, COLL, 512>(map, a, fullbc, rows, box, err, s);
  return launch_tma_pair_pitch<L, SK, COLL, 1024>(map, a, fullbc, rows, box, err, s);
}

}  // namespace xlbg
