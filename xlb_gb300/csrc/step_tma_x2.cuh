// TMA-staged step with two cells per consumer thread and packed FP32 arithmetic,
// for pair-form BGK (XLBG_BGK_PAIR) with the shifted 16-bit stores (FP16S, BF16S).
//
// Consumer thread t owns the adjacent cells z0 = 2t and z1 = 2t + 1 of every
// staged row.  When both are fluid cells (bc id 0) their populations are
// decoded into f32x2 registers (lane 0: z0, lane 1: z1), collided with the
// packed instructions fma/add/sub/mul.rn.f32x2, encoded two at a time
// (cvt.rn.f16x2.f32 / cvt.rn.bf16x2.f32) and stored as one 32-bit word per
// direction.  Each packed instruction rounds each lane exactly like its scalar
// form, and the operations are those of bgk_pair's FP32 branch in the same
// order, so the results equal the one-cell kernel's bit for bit.  A pair with a
// boundary or skipped cell runs cell_update on each of its cells.
//
// The producer warp and the stage hand-off are step_kernel_tma's.  Selected with
// XLBG_TMA_X2=1 only: with half the consumer warps per SM it ran about 5 %
// slower than the one-cell kernel (see tma_x2_enabled).
#pragma once

#include "step_tma.cuh"

namespace xlbg {
namespace x2 {

// Two FP32 lanes in one 64-bit register pair.
struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 mk(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ f2 splat(float x) { return mk(x, x); }
__device__ __forceinline__ void split(f2 a, float& l, float& h) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(l), "=f"(h) : "l"(a.v));
}
__device__ __forceinline__ float lo(f2 a) {
  float l, h;
  split(a, l, h);
  (void)h;
  return l;
}
__device__ __forceinline__ float hi(f2 a) {
  float l, h;
  split(a, l, h);
  (void)l;
  return h;
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 fma(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// Packed forms of Store<SK, float>::dec / enc for the shifted 16-bit stores.
template <int SK>
struct Codec;

template <>
struct Codec<SK_F16S> {
  using St = Store<SK_F16S, float>;
  __device__ static __forceinline__ f2 dec(unsigned short b0, unsigned short b1, float w) {
    return fma(mk(__half2float(__ushort_as_half(b0)), __half2float(__ushort_as_half(b1))), splat(St::kInvScale),
               splat(w));
  }
  __device__ static __forceinline__ unsigned enc(f2 v, float w) {
    const f2 s = fma(v, splat(St::kScale), splat(-(w * St::kScale)));
    unsigned r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi(s)), "f"(lo(s)));
    return r;
  }
};

template <>
struct Codec<SK_BF16S> {
  __device__ static __forceinline__ f2 dec(unsigned short b0, unsigned short b1, float w) {
    return mk(__uint_as_float((unsigned)b0 << 16), __uint_as_float((unsigned)b1 << 16)) + splat(w);
  }
  __device__ static __forceinline__ unsigned enc(f2 v, float w) {
    const f2 s = v - splat(w);
    unsigned r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi(s)), "f"(lo(s)));
    return r;
  }
};

// bgk_pair's FP32 branch (physics.cuh) on two cells: the same operations in the
// same order, including the additions to zero that start rho's partner sums.
template <class L, int P>
__device__ __forceinline__ void pair_moments(const f2 (&f)[L::Q], f2& rho, f2 (&j)[L::D]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    const f2 sig = f[l] + f[o];
    const f2 dif = f[l] - f[o];
    rho = rho + sig;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) j[d] = j[d] + dif;
      if (L::c(l, d) == -1) j[d] = j[d] - dif;
    }
    pair_moments<L, P + 1>(f, rho, j);
  }
}

template <class L, int P>
__device__ __forceinline__ void pair_update(const f2 (&f)[L::Q], const f2 (&u)[L::D], f2 base, f2 omf, f2 orho,
                                            f2 (&fo)[L::Q]) {
  if constexpr (P < (L::Q - 1) / 2) {
    constexpr int l = pair_at<L>(P);
    constexpr int o = opp<L>(l);
    f2 cu = splat(0.0f);
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(l, d) == 1) cu = cu + u[d];
      if (L::c(l, d) == -1) cu = cu - u[d];
    }
    // t per lane: with t = 3 cu as a packed multiply feeding the packed e + t and
    // e - t, results differed from the separately rounded operations in about 4 %
    // of the outputs (measured on sm_103a with CUDA 13.0, the pair behaving as a
    // fused multiply-add); with t per lane they are equal bit for bit
    const f2 t = mk(3.0f * lo(cu), 3.0f * hi(cu));
    const f2 ow = orho * splat((float)weight<L>(l));
    const f2 e = fma(splat(4.5f) * cu, cu, base);
    fo[l] = fma(omf, f[l], ow * (e + t));
    fo[o] = fma(omf, f[o], ow * (e - t));
    pair_update<L, P + 1>(f, u, base, omf, orho, fo);
  }
}

template <class L>
__device__ __forceinline__ void bgk_pair(const f2 (&f)[L::Q], float omega, f2 (&fo)[L::Q]) {
  f2 rho = f[0];
  f2 j[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) j[d] = splat(0.0f);
  pair_moments<L, 0>(f, rho, j);
  const f2 inv = mk(1.0f / lo(rho), 1.0f / hi(rho));
  f2 u[L::D];
#pragma unroll
  for (int d = 0; d < L::D; ++d) u[d] = j[d] * inv;
  f2 usq = u[0] * u[0];
#pragma unroll
  for (int d = 1; d < L::D; ++d) usq = fma(u[d], u[d], usq);
  const f2 base = fma(splat(-1.5f), usq, splat(1.0f));
  const f2 omf = splat(1.0f - omega);
  const f2 orho = splat(omega) * rho;
  fo[0] = fma(omf, f[0], orho * splat((float)weight<L>(0)) * base);
  pair_update<L, 0>(f, u, base, omf, orho, fo);
}

}  // namespace x2

template <int PITCH>
__host__ __device__ constexpr int tma_x2_consumers() {
  return PITCH / 2;
}

template <int PITCH>
__host__ __device__ constexpr int tma_x2_min_blocks() {
  return PITCH <= 256 ? 4 : (PITCH == 512 ? 2 : 1);
}

// Same tensor map, grid, shared memory and hand-off as step_kernel_tma; PITCH / 2
// consumers plus the producer warp.  n2 even (the host requires n2 % 8 == 0).
template <class L, int SK, bool FULLBC, int PITCH>
__global__ void __launch_bounds__(tma_x2_consumers<PITCH>() + 32, tma_x2_min_blocks<PITCH>())
    step_kernel_tma_x2(const __grid_constant__ CUtensorMap map, const StepArgs a, int rows, int box, int* err) {
  using C = x2::Codec<SK>;
  using x2::f2;
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned ROW = PITCH * 2;
  constexpr unsigned STAGE = Q * ROW;
  constexpr int CT = tma_x2_consumers<PITCH>();
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
  if (base % 128 != 0) {  // tensor copies need an aligned destination: report, copy nothing
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
    tma_produce<L, PITCH>(map, base, full, empty, tid - CT, i0, r0, nr, n0, n1, n2, box, err);
    return;
  }

  // ---- consumers: cells z0 = 2 tid and z0 + 1 of every row ----
  const int lane = tid & 31;
  const int z0 = 2 * tid;
  const bool active = z0 < n2;
  // byte offsets in a staged row of each cell's source element for c2 = -1, 0, +1
  const unsigned zb0[3] = {(unsigned)(z0 + 1) * 2, (unsigned)z0 * 2, (unsigned)(z0 == 0 ? n2 - 1 : z0 - 1) * 2};
  const unsigned zb1[3] = {(unsigned)(z0 + 2 == n2 ? 0 : z0 + 2) * 2, (unsigned)(z0 + 1) * 2, (unsigned)z0 * 2};
  double dm = 0.0, df[3] = {0.0, 0.0, 0.0};
  const unsigned row0 = ((unsigned)i0 * (unsigned)n1 + (unsigned)r0) * (unsigned)n2 + (unsigned)z0;
  // the two bc ids run one row ahead, so their load latency hides behind a row's work
  const unsigned short skip2 = 0xffff;
  unsigned short ids_next =
      (active && nr > 0) ? *reinterpret_cast<const unsigned short*>(a.bc_mask + row0) : skip2;
  const float omega = omega_of<float>(a);
  const size_t plane = (size_t)a.ncell;
  for (int k = 0; k < nr; ++k) {
    const unsigned s = (unsigned)(k % S);
    const int y = r0 + k;
    const unsigned cell = row0 + (unsigned)k * (unsigned)n2;
    const unsigned short ids = ids_next;
    if (k + 1 < nr)
      ids_next = active ? *reinterpret_cast<const unsigned short*>(a.bc_mask + cell + (unsigned)n2) : skip2;
    const bool ok = mbar_wait(full + 8 * s, (unsigned)((k / S) & 1), kTmaWaitNs);
    if (__any_sync(0xffffffffu, !ok)) {  // the stage never completed: report, store nothing
      if (lane == 0) atomicAdd(err, 1);
      return;
    }
    f2 f[Q];
    if (active) {
      const unsigned char* st = smem + s * STAGE;
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        const int c = axis_c<L>(l, 2) + 1;
        unsigned short b0, b1;
        if (c == 1) {  // unshifted: both cells' sources in one aligned word
          const unsigned w = *reinterpret_cast<const unsigned*>(st + l * ROW + zb0[1]);
          b0 = (unsigned short)(w & 0xffffu);
          b1 = (unsigned short)(w >> 16);
        } else {
          b0 = *reinterpret_cast<const unsigned short*>(st + l * ROW + zb0[c]);
          b1 = *reinterpret_cast<const unsigned short*>(st + l * ROW + zb1[c]);
        }
        f[l] = C::dec(b0, b1, (float)weight<L>(l));
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + 8 * s);
    if (!active || ids == skip2) continue;
    if (ids == 0) {
      f2 fo[Q];
      x2::bgk_pair<L>(f, omega, fo);
      unsigned* out = reinterpret_cast<unsigned*>(static_cast<unsigned short*>(a.f1) + cell);
#pragma unroll
      for (int l = 0; l < Q; ++l) out[(size_t)l * (plane / 2)] = C::enc(fo[l], (float)weight<L>(l));
      continue;
    }
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      const uint8_t id = (uint8_t)(h ? ids >> 8 : ids & 0xff);
      if (id == 255) continue;
      float fh[Q];
#pragma unroll
      for (int l = 0; l < Q; ++l) fh[l] = h ? x2::hi(f[l]) : x2::lo(f[l]);
      cell_update<L, SK, float, 2, FULLBC, false>(a, i0, y, z0 + h, cell + (unsigned)h, id, fh, dm, df);
    }
  }
}

template <class L, int SK, int PITCH>
int launch_tma_x2_pitch(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                        cudaStream_t s) {
  const unsigned smem = tma_smem_bytes<L, PITCH>();
  static const bool attr_full = cudaFuncSetAttribute(step_kernel_tma_x2<L, SK, true, PITCH>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
  static const bool attr_part = cudaFuncSetAttribute(step_kernel_tma_x2<L, SK, false, PITCH>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
  if (!attr_full || !attr_part) return (int)cudaErrorInvalidValue;
  const dim3 grid((unsigned)a.n0, (unsigned)((a.n1 + rows - 1) / rows));
  const unsigned threads = tma_x2_consumers<PITCH>() + 32;
  if (fullbc)
    step_kernel_tma_x2<L, SK, true, PITCH><<<grid, threads, smem, s>>>(map, a, rows, box, err);
  else
    step_kernel_tma_x2<L, SK, false, PITCH><<<grid, threads, smem, s>>>(map, a, rows, box, err);
  return (int)cudaGetLastError();
}

template <int LAT, int SK>
int launch_tma_x2_t(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                    cudaStream_t s) {
  using L = Lattice<LAT>;
  if (a.n2 <= 256) return launch_tma_x2_pitch<L, SK, 256>(map, a, fullbc, rows, box, err, s);
  if (a.n2 <= 512) return launch_tma_x2_pitch<L, SK, 512>(map, a, fullbc, rows, box, err, s);
  return launch_tma_x2_pitch<L, SK, 1024>(map, a, fullbc, rows, box, err, s);
}

}  // namespace xlbg
