// Fused step with TMA row staging, one cell per consumer thread: raw FP16
// stores with XLB-order BGK, and FP32 D3Q27 KBC (plain and with the fused
// diagnostics).  The shifted 16-bit stores use the segmented two-cell kernel of
// step_tma_seg.cuh, which shares the ring, the producer hand-off and the
// bounded waits defined here.
//
// The marching kernel keeps each warp's next 19 loads behind its current
// collision, so with 16-bit populations (half the bytes per cell of FP32) it
// runs out of bytes in flight before it runs out of bandwidth.  Here the pulls
// are tensor copies (cp.async.bulk.tensor) issued by one thread into a ring of
// shared-memory stages, completed on mbarriers:
//
//   CTA = one plane i0 of axis 0 and a band of rows of axis 1; one thread per
//         cell of the contiguous axis (n2 <= PITCH threads) plus a producer warp
//         that issues the copies.
//   stage = for each direction l, the full source row (i0 - c0_l, i1 - c1_l) of
//         plane l, both wrapped as the stream wraps (stream.py:64-82): Q rows of
//         PITCH store values.  The contiguous-axis shift and its wrap are a
//         shared-memory index: thread i2 reads element (i2 - c2_l) mod n2.
//   ring  = S stages; stage s holds row k while rows k+1 .. k+S-1 are in flight.
//
// Each source element is copied once (every direction reads its own plane), so
// DRAM traffic stays at the algorithmic Q * 2 bytes per cell.  After the pull,
// the per-cell work is cell_update's, unchanged, so results are bit-identical
// to the marching kernel.
//
// Every wait is bounded: a stage that does not complete within one second
// (%globaltimer) makes the block count itself in *err, wait (bounded) for its
// other copies in flight and return without storing.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include <type_traits>

#include "step_kernel.cuh"

namespace xlbg {

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// One try_wait (the hardware suspends the thread for a bounded time inside it).
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: false when the phase has not completed within limit_ns.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// 4D tiled tensor copy global -> shared, completing on an mbarrier.  c0 (the
// contiguous-axis coordinate) is 0 or a multiple of 256 elements here, so the
// 16-byte rule on the innermost coordinate holds.
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

constexpr int kTmaBox = 256;            // contiguous-axis elements per tensor copy (at most)
constexpr unsigned long long kTmaWaitNs = 1000000000ull;  // bounded mbarrier wait: one second

template <class L>
__host__ __device__ constexpr int tma_stages() {
  return L::Q <= 19 ? 5 : 3;
}

// Consumer threads of a block: one per staged element (PITCH <= 512).
template <int PITCH>
__host__ __device__ constexpr int tma_consumers() {
  return PITCH;
}

// CTAs per SM the launch bounds ask for (consumers + one producer warp): 16-bit
// BGK, whose cells need few registers, as many as the shared memory allows;
// 4-byte stores (KBC) one: asking for two capped KBC at 96 registers with
// spills, while its ~128 registers still fit two 224-thread CTAs (PITCH 192).
template <int EB, int PITCH>
__host__ __device__ constexpr int tma_min_blocks() {
  return EB == 2 ? (PITCH <= 256 ? 4 : 2) : 1;
}

// shared memory: S stages of Q rows of EB-byte elements, then S "full" and S "empty" mbarriers
template <class L, int EB, int PITCH>
__host__ __device__ constexpr unsigned tma_smem_bytes() {
  return (unsigned)tma_stages<L>() * L::Q * PITCH * EB + 16u * tma_stages<L>();
}

// Producer warp of a TMA-staged step CTA: lane l < Q issues the copies of
// direction l, row after row, into the S-stage ring at base (see the hand-off
// described at step_kernel_tma).  A bounded wait that runs out counts one
// fault, lets the copies still in flight land and returns.
template <class L, int EB, int PITCH>
__device__ __forceinline__ void tma_produce(const CUtensorMap& map, unsigned base, unsigned full, unsigned empty, int l,
                                            int i0, int r0, int nr, int n0, int n1, int n2, int box, int* err) {
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned ROW = PITCH * EB;
  constexpr unsigned STAGE = Q * ROW;
  const bool issuer = l < Q;
  const int nbox = (n2 + box - 1) / box;
  const unsigned tx_bytes = (unsigned)(Q * nbox * box * EB);
  const int c0 = issuer ? axis_c<L>(l, 0) : 0, c1 = issuer ? axis_c<L>(l, 1) : 0;
  const int xs = c0 == 1 ? (i0 == 0 ? n0 - 1 : i0 - 1) : (c0 == -1 ? (i0 == n0 - 1 ? 0 : i0 + 1) : i0);
  for (int k = 0; k < nr; ++k) {
    const unsigned s = (unsigned)(k % S);
    const int u = k / S;
    const bool ok = u == 0 || mbar_wait(empty + 8 * s, (unsigned)((u - 1) & 1), kTmaWaitNs);
    if (__any_sync(0xffffffffu, !ok)) {
      // consumers stopped: report, let the copies still in flight land
      if (l == 0) {
        atomicAdd(err, 1);
        for (int j = k - S + 1; j < k; ++j)
          if (j >= 0) mbar_wait(full + 8 * (j % S), (unsigned)((j / S) & 1), kTmaWaitNs);
      }
      return;
    }
    const unsigned bar = full + 8 * s;
    if (l == 0) mbar_expect_tx(bar, tx_bytes);
    __syncwarp();
    if (issuer) {
      const int y = r0 + k;
      const int ys = c1 == 1 ? (y == 0 ? n1 - 1 : y - 1) : (c1 == -1 ? (y == n1 - 1 ? 0 : y + 1) : y);
      for (int b = 0; b < nbox; ++b)
        tma_load_4d(base + s * STAGE + (unsigned)l * ROW + b * box * EB, &map, b * box, ys, xs, l, bar);
    }
  }
}

// map: 4D tensor map of f0 as (n2, n1, n0, Q) elements of the store (2 or 4
// bytes), box (box, 1, 1, 1) with box = min(n2, 256).  Grid: (n0, ceil(n1 /
// rows)); CT + 32 threads per block, CT = tma_consumers<PITCH>(): CT consumers
// (thread i2 owns cell i2 of every row) and one producer warp, whose lanes issue
// the copies.  Staged rows hold PITCH elements; n2 <= CT, n2 * element bytes a
// multiple of 16; cell offsets fit 31 bits (the host checks).  DIAG: the
// diagnostics step (mass of the output, force on the input, as the marching
// kernel's): per-thread FP64 sums, reduced over each consumer warp by shuffles
// and added to the slot array by lane 0 (no block barrier: the producer warp
// has left).  Plane offsets: the fluid path stores through the cell's slot in
// plane 0 plus 64-bit plane offsets at any size; the boundary paths index
// f0 / f1 planes with Idx, 32-bit unsigned when Q * cells < 2^32 and 64-bit
// (WIDE) above.
//
// Hand-off per stage s (row k, use u = k / S):
//   producer: wait empty[s] phase u - 1 (u > 0); lane 0 posts expect_tx on
//             full[s], then lane l < Q issues the copies of direction l
//   consumer warp: wait full[s] phase u, read its cells, __syncwarp, lane 0
//                  arrives on empty[s] (CT / 32 arrivals complete the phase)
// No block-wide barrier after set-up: consumer warps drift up to S rows apart.
template <class L, int SK, int COLL, bool FULLBC, int PITCH, bool WIDE, bool DIAG = false>
__global__ void __launch_bounds__(tma_consumers<PITCH>() + 32,
                                  tma_min_blocks<sizeof(typename Store<SK, float>::Bits), PITCH>())
    step_kernel_tma(const __grid_constant__ CUtensorMap map, const StepArgs a, int rows, int box, int* err) {
  using T = float;
  using Idx = typename std::conditional<WIDE, long long, unsigned>::type;
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int EB = sizeof(Bits);
  static_assert(EB == 2 || EB == 4, "16- or 32-bit stores");
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned ROW = PITCH * EB;
  constexpr unsigned STAGE = Q * ROW;
  constexpr int CT = tma_consumers<PITCH>();
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
    tma_produce<L, EB, PITCH>(map, base, full, empty, tid - CT, i0, r0, nr, n0, n1, n2, box, err);
    return;
  }

  // ---- consumers ----
  const int lane = tid & 31;
  const int i2 = tid;
  const bool active = i2 < n2;
  // byte offset in a staged row of the source element for c2 = -1, 0, +1
  const unsigned zb[3] = {(unsigned)(i2 == n2 - 1 ? 0 : i2 + 1) * EB, (unsigned)i2 * EB,
                          (unsigned)(i2 == 0 ? n2 - 1 : i2 - 1) * EB};
  double dm = 0.0, df[3] = {0.0, 0.0, 0.0};
  // the bc ids run one row ahead, so their load latency hides behind a row's collision
  const unsigned row0 = ((unsigned)i0 * (unsigned)n1 + (unsigned)r0) * (unsigned)n2 + (unsigned)i2;
  uint8_t id_next = (active && nr > 0) ? a.bc_mask[row0] : (uint8_t)255;
  for (int k = 0; k < nr; ++k) {
    const unsigned s = (unsigned)(k % S);
    const int y = r0 + k;
    const unsigned cell = row0 + (unsigned)k * (unsigned)n2;
    const uint8_t id = id_next;
    if (k + 1 < nr) id_next = active ? a.bc_mask[cell + (unsigned)n2] : (uint8_t)255;
    const bool ok = mbar_wait(full + 8 * s, (unsigned)((k / S) & 1), kTmaWaitNs);
    if (__any_sync(0xffffffffu, !ok)) {  // the stage never completed: report, store nothing
      if (lane == 0) atomicAdd(err, 1);
      return;
    }
    T f[Q];
    if (active) {
      const unsigned char* st = smem + s * STAGE;
#pragma unroll
      for (int l = 0; l < Q; ++l)
        f[l] = load_pop<SK, T, COLL>(*reinterpret_cast<const Bits*>(st + l * ROW + zb[axis_c<L>(l, 2) + 1]),
                                     T(weight<L>(l)));
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + 8 * s);
    if (COLL != 1 && __all_sync(0xffffffffu, id == 0)) {
      // every cell of the warp is fluid (lanes past the row carry id 255): the
      // collision and the store alone, which is what cell_update does for id 0
      // (BGK forms only: a second inlined copy of the large KBC collision
      // measured slower)
      T fo[Q];
      collide<L, SK, T, COLL>(f, omega_of<T>(a), fo);
      double dmc = 0.0;
      store_cell_u32<L, SK, T, COLL, DIAG>(a, cell, fo, dmc);
      if constexpr (DIAG) dm += dmc;
    } else if constexpr (DIAG) {
      if (id != 255) {
        double dmc = 0.0, dfc[3] = {0.0, 0.0, 0.0};
        cell_update<L, SK, T, COLL, FULLBC, true>(a, i0, y, i2, (Idx)cell, id, f, dmc, dfc);
        dm += dmc;
        df[0] += dfc[0];
        df[1] += dfc[1];
        df[2] += dfc[2];
      }
    } else {
      if (id != 255) cell_update<L, SK, T, COLL, FULLBC, false>(a, i0, y, i2, (Idx)cell, id, f, dm, df);
    }
  }
  if constexpr (DIAG) {
    double v[4] = {dm, df[0], df[1], df[2]};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    }
    if (lane == 0) {
      const unsigned slot = ((blockIdx.x * gridDim.y + blockIdx.y) * CONSUMER_WARPS + (tid >> 5)) % kDiagSlots;
#pragma unroll
      for (int k = 0; k < 4; ++k) atomicAdd(a.diag_slots + slot * 4 + k, v[k]);
    }
  }
}

// Launch for one (lattice, store, collision): picks the pitch, sets the shared
// memory size once per instantiation.  Returns the CUDA error of the launch.
template <class L, int SK, int COLL, bool FULLBC, int PITCH, bool WIDE, bool DIAG>
int launch_tma_kernel(const CUtensorMap& map, const StepArgs& a, int rows, int box, int* err, cudaStream_t s) {
  constexpr int EB = sizeof(typename Store<SK, float>::Bits);
  const unsigned smem = tma_smem_bytes<L, EB, PITCH>();
  static const bool attr = cudaFuncSetAttribute(step_kernel_tma<L, SK, COLL, FULLBC, PITCH, WIDE, DIAG>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
  if (!attr) return (int)cudaErrorInvalidValue;
  const dim3 grid((unsigned)a.n0, (unsigned)((a.n1 + rows - 1) / rows));
  step_kernel_tma<L, SK, COLL, FULLBC, PITCH, WIDE, DIAG>
      <<<grid, tma_consumers<PITCH>() + 32, smem, s>>>(map, a, rows, box, err);
  return (int)cudaGetLastError();
}

// The BC code variant (fullbc), the diagnostics step (a.diag_slots set; always
// with the full BC code) when the instantiation has it (WITH_DIAG), and the
// plane-offset width (a.wide).
template <class L, int SK, int COLL, int PITCH, bool WIDE, bool WITH_DIAG>
int launch_tma_variant(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                       cudaStream_t s) {
  if constexpr (WITH_DIAG) {
    if (a.diag_slots != nullptr) return launch_tma_kernel<L, SK, COLL, true, PITCH, WIDE, true>(map, a, rows, box, err, s);
  }
  if (fullbc) return launch_tma_kernel<L, SK, COLL, true, PITCH, WIDE, false>(map, a, rows, box, err, s);
  return launch_tma_kernel<L, SK, COLL, false, PITCH, WIDE, false>(map, a, rows, box, err, s);
}

template <class L, int SK, int COLL, int PITCH, bool WITH_DIAG>
int launch_tma_pitch(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                     cudaStream_t s) {
  return a.wide ? launch_tma_variant<L, SK, COLL, PITCH, true, WITH_DIAG>(map, a, fullbc, rows, box, err, s)
                : launch_tma_variant<L, SK, COLL, PITCH, false, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
}

// Staged-row width for a contiguous axis of n2 <= 512 cells: 16-bit stores 256
// or 512, 4-byte stores 192, 256 or 512.
template <int EB>
inline int tma_pitch_for(int n2) {
  if (EB == 4) return n2 <= 192 ? 192 : (n2 <= 256 ? 256 : 512);
  return n2 <= 256 ? 256 : 512;
}

template <int LAT, int SK, int COLL, bool WITH_DIAG = false>
int launch_tma_t(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                 cudaStream_t s) {
  using L = Lattice<LAT>;
  constexpr int EB = sizeof(typename Store<SK, float>::Bits);
  const int pitch = tma_pitch_for<EB>(a.n2);
  if constexpr (EB == 4) {
    if (pitch == 192) return launch_tma_pitch<L, SK, COLL, 192, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
    if (pitch == 256) return launch_tma_pitch<L, SK, COLL, 256, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
    return launch_tma_pitch<L, SK, COLL, 512, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
  } else {
    if (pitch == 256) return launch_tma_pitch<L, SK, COLL, 256, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
    return launch_tma_pitch<L, SK, COLL, 512, WITH_DIAG>(map, a, fullbc, rows, box, err, s);
  }
}

// Per-lattice entry points (step_tma_*.cu): raw FP16 with XLB-order BGK (code
// 0); other combinations return -1 (the shifted stores take the segmented
// kernel of step_tma_seg.cuh).
template <int LAT>
int launch_tma_lattice(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows, int box,
                       int* err, cudaStream_t s) {
  if (sk == SK_F16 && coll == 0) return launch_tma_t<LAT, SK_F16, 0>(map, a, fullbc, rows, box, err, s);
  return -1;
}

int launch_step_tma_d2q9(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows,
                         int box, int* err, cudaStream_t s);
int launch_step_tma_d3q19(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows,
                          int box, int* err, cudaStream_t s);
int launch_step_tma_d3q27(const CUtensorMap& map, const StepArgs& a, int sk, int coll, bool fullbc, int rows,
                          int box, int* err, cudaStream_t s);
// Segmented two-cell kernel (step_tma_seg.cuh): shifted 16-bit stores, codes 3
// and 4; blocks own kSeg cells of the contiguous axis.
constexpr int kSeg = 256;
int launch_step_seg_d2q9(const StepArgs& a, int sk, int coll, bool fullbc, bool diag, int nseg, int rows, int* err,
                         cudaStream_t s);
int launch_step_seg_d3q19(const StepArgs& a, int sk, int coll, bool fullbc, bool diag, int nseg, int rows, int* err,
                          cudaStream_t s);
int launch_step_seg_d3q27(const StepArgs& a, int sk, int coll, bool fullbc, bool diag, int nseg, int rows, int* err,
                          cudaStream_t s);
// FP32 store, KBC, D3Q27, with the diagnostics step (step_tma_d3q27_kbc.cu).
int launch_step_tma_d3q27_kbc32(const CUtensorMap& map, const StepArgs& a, bool fullbc, int rows, int box, int* err,
                                cudaStream_t s);

}  // namespace xlbg
