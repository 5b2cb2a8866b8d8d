// Segmented two-cell step for the shifted 16-bit stores (collision codes 3 and
// 4) on rows of any length that is a multiple of 8 cells.
//
// CTA = one segment of at most kSeg = 256 cells of the contiguous axis, for a
// band of rows of one plane: 128 consumer threads (two cells each, the packed
// collision of pair_collide.cuh) and a producer warp; four CTAs a SM (96
// registers, 51 KB of shared memory for D3Q19).  Short CTAs keep 16 consumer
// warps on every SM whatever the row length: staging whole rows instead needs
// a 1024-cell stage for rows of 513..1024 cells, one CTA a SM, and measured
// 51 GLUPS at 1024 x 1024 x 768 against 80 here (D3Q19 FP16S; at 512^3 the
// whole-row two-cell kernel gave 77.9 GLUPS and this one 82.6).
//
// Staged row of direction l (544 bytes):
//   [8-cell left apron | kSeg cells of the segment | 8-cell right apron]
// holding source element z (segment-local, -1 .. seglen) at byte 16 + 2 z, so
// a consumer reads the element its cell pulls at a fixed offset with no wrap
// test.  Only the apron a direction pulls from is filled: c_z = +1 reads cell
// z0 - 1, c_z = -1 cell z0 + seglen.  The producer's lane l copies, per row,
// one run of the source row with untiled bulk copies (cp.async.bulk): the
// segment extended by the 8-cell apron where the neighbour cell lies inside
// the row, and at the two ends of the axis a separate 16-byte copy of the
// other end's 8 cells (the periodic wrap of the pull, stream.py:64-82).
// Every run starts and ends on a 16-byte boundary (n2, z0 and seglen are
// multiples of 8 cells, f0 is 16-byte aligned, so plane and row offsets are
// too), which is all an untiled bulk copy asks.  Consecutive blocks are the
// segments of one (plane, band), so a segment's aprons are read from L2 while
// its neighbours stage the same rows.
//
// The source rows of a direction are its own plane's rows (i0 - c0_l, i1 -
// c1_l), wrapped as the stream wraps, so each source element is copied once
// (plus the 16-byte aprons) and DRAM traffic stays at the algorithmic Q * 2
// bytes read per cell.  Every wait is bounded: a stage that does not complete
// within one second (%globaltimer) makes the block count itself in *err, wait
// (bounded) for its other copies in flight and return without storing.
#pragma once
#include "pair_collide.cuh"
#include "step_tma.cuh"

namespace xlbg {

constexpr int kSegConsumers = kSeg / 2;      // consumer threads: two cells each
constexpr unsigned kSegRow = 2 * kSeg + 32;  // staged row bytes: segment plus two 16-byte aprons

// Number of directions whose pull crosses cells along the contiguous axis
// (each adds one 16-byte apron to a stage).
template <class L>
__host__ __device__ constexpr int seg_apron_dirs() {
  int n = 0;
  for (int l = 0; l < L::Q; ++l) n += axis_c<L>(l, 2) != 0 ? 1 : 0;
  return n;
}

template <class L>
__host__ __device__ constexpr unsigned seg_smem_bytes() {
  return (unsigned)tma_stages<L>() * L::Q * kSegRow + 16u * tma_stages<L>();
}

// Untiled bulk copy global -> shared completing on an mbarrier; dst, src and
// bytes multiples of 16.
__device__ __forceinline__ void bulk_load(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Producer warp of a segment CTA: lane l < Q copies direction l's run (and its
// wrapped apron at an end of the axis) of every row into the ring.  A bounded
// wait that runs out counts one fault, lets the copies in flight land and returns.
template <class L>
__device__ __forceinline__ void seg_produce(const StepArgs& a, unsigned base, unsigned full, unsigned empty, int l,
                                            int i0, int z0, int seglen, int r0, int nr, int* err) {
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned STAGE = Q * kSegRow;
  const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
  const bool issuer = l < Q;
  const unsigned tx_bytes = (unsigned)(Q * 2 * seglen + 16 * seg_apron_dirs<L>());
  const int c0 = issuer ? axis_c<L>(l, 0) : 0, c1 = issuer ? axis_c<L>(l, 1) : 0;
  const int c2 = issuer ? axis_c<L>(l, 2) : 0;
  const int xs = c0 == 1 ? (i0 == 0 ? n0 - 1 : i0 - 1) : (c0 == -1 ? (i0 == n0 - 1 ? 0 : i0 + 1) : i0);
  const int end = z0 + seglen;
  // the run [lo, hi) of the source row, landing at row byte 16 + 2 (lo - z0)
  const int lo = (c2 == 1 && z0 > 0) ? z0 - 8 : z0;
  const int hi = (c2 == -1 && end < n2) ? end + 8 : end;
  const unsigned run_dst = (unsigned)(16 + 2 * (lo - z0));
  const unsigned run_bytes = (unsigned)(2 * (hi - lo));
  // the apron that wraps: cells n2 - 8 .. n2 - 1 to the left of z = 0, cells 0 .. 7 to the right of n2 - 1
  const bool wrap = (c2 == 1 && z0 == 0) || (c2 == -1 && end == n2);
  const int wrap_src = c2 == 1 ? n2 - 8 : 0;
  const unsigned wrap_dst = c2 == 1 ? 0u : (unsigned)(16 + 2 * seglen);
  const uint16_t* plane = static_cast<const uint16_t*>(a.f0) + (size_t)(issuer ? l : 0) * (size_t)a.ncell;
  for (int k = 0; k < nr; ++k) {
    const unsigned s = (unsigned)(k % S);
    const int u = k / S;
    const bool ok = u == 0 || mbar_wait(empty + 8 * s, (unsigned)((u - 1) & 1), kTmaWaitNs);
    if (__any_sync(0xffffffffu, !ok)) {
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
      const uint16_t* src = plane + ((size_t)xs * (size_t)n1 + (size_t)ys) * (size_t)n2;
      const unsigned row = base + s * STAGE + (unsigned)l * kSegRow;
      bulk_load(row + run_dst, src + lo, run_bytes, bar);
      if (wrap) bulk_load(row + wrap_dst, src + wrap_src, 16u, bar);
    }
  }
}

// Grid: (n0 * nseg, ceil(n1 / rows)), block kSegConsumers + 32 threads,
// seg_smem_bytes<L>() of dynamic shared memory; block x = i0 * nseg + segment.
// n2 a multiple of 8, cell offsets fit 31 bits, f0 16-byte aligned, bc_mask
// 2-byte and f1 4-byte aligned (the host checks).  DIAG: the diagnostics step
// (mass of the output as stored, force on the input, as the one-cell kernels
// define them): per-thread FP64 sums, reduced over each consumer warp by
// shuffles and added to the slot array by lane 0.
template <class L, int SK, int COLL, bool FULLBC, bool WIDE, bool DIAG>
// (three CTAs a SM for DIAG: capped at 96 registers for four, it spilled)
__global__ void __launch_bounds__(kSegConsumers + 32, DIAG ? 3 : 4)
    step_kernel_seg(const StepArgs a, int nseg, int rows, int* err) {
  using St = Store<SK, float>;
  using Bits = typename St::Bits;
  static_assert(sizeof(Bits) == 2, "16-bit stores");
  static_assert(COLL == 3 || COLL == 4, "BGK on deviations");
  constexpr int Q = L::Q;
  constexpr int S = tma_stages<L>();
  constexpr unsigned STAGE = Q * kSegRow;
  constexpr unsigned CONSUMER_WARPS = kSegConsumers / 32;
  extern __shared__ __align__(1024) unsigned char smem[];
  const unsigned base = smem_addr(smem);
  const unsigned full = base + S * STAGE;
  const unsigned empty = full + 8 * S;
  const int n1 = a.n1, n2 = a.n2;
  const int i0 = (int)(blockIdx.x / (unsigned)nseg);
  const int z0 = (int)(blockIdx.x - (unsigned)i0 * (unsigned)nseg) * kSeg;
  const int seglen = min(kSeg, n2 - z0);
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

  if (tid >= kSegConsumers) {
    seg_produce<L>(a, base, full, empty, tid - kSegConsumers, i0, z0, seglen, r0, nr, err);
    return;
  }

  // ---- consumers: segment cells p = 2 tid and 2 tid + 1 of every row ----
  const int lane = tid & 31;
  const int p0 = 2 * tid;
  const bool active = p0 < seglen;  // seglen is even: both cells or neither
  double dm = 0.0, df[3] = {0.0, 0.0, 0.0};
  const unsigned row0 = ((unsigned)i0 * (unsigned)n1 + (unsigned)r0) * (unsigned)n2 + (unsigned)(z0 + p0);
  uint16_t ids_next =
      (active && nr > 0) ? *reinterpret_cast<const uint16_t*>(a.bc_mask + row0) : (uint16_t)0xffff;
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
      // element z of direction l's row at byte 16 + 2 z: cell p pulls z = p - c_z
      const unsigned char* st = smem + s * STAGE + 16 + 2 * p0;
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        const int cz = axis_c<L>(l, 2);
        float ga, gb;
        if (cz == 0) {
          const uint32_t w = *reinterpret_cast<const uint32_t*>(st + l * kSegRow);
          ga = St::dev((Bits)(w & 0xffffu), 0.0f);
          gb = St::dev((Bits)(w >> 16), 0.0f);
        } else {
          ga = St::dev(*reinterpret_cast<const Bits*>(st + l * kSegRow - 2 * cz), 0.0f);
          gb = St::dev(*reinterpret_cast<const Bits*>(st + l * kSegRow + 2 - 2 * cz), 0.0f);
        }
        g[l] = pk2(ga, gb);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + 8 * s);
    pair_finish<L, SK, COLL, FULLBC, WIDE, DIAG>(a, g, ids, i0, y, z0 + p0, cell, dm, df);
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

template <class L, int SK, int COLL, bool FULLBC, bool WIDE, bool DIAG>
int launch_seg_kernel(const StepArgs& a, int nseg, int rows, int* err, cudaStream_t s) {
  const unsigned smem = seg_smem_bytes<L>();
  static const bool attr = cudaFuncSetAttribute(step_kernel_seg<L, SK, COLL, FULLBC, WIDE, DIAG>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
  if (!attr) return (int)cudaErrorInvalidValue;
  const dim3 grid((unsigned)a.n0 * (unsigned)nseg, (unsigned)((a.n1 + rows - 1) / rows));
  step_kernel_seg<L, SK, COLL, FULLBC, WIDE, DIAG><<<grid, kSegConsumers + 32, smem, s>>>(a, nseg, rows, err);
  return (int)cudaGetLastError();
}

// The diagnostics step always runs with the full BC code (the force BC's cells
// go through it), so DIAG is instantiated with FULLBC only.
template <int LAT, int SK, int COLL>
int launch_seg_t(const StepArgs& a, bool fullbc, bool diag, int nseg, int rows, int* err, cudaStream_t s) {
  using L = Lattice<LAT>;
  if (diag)
    return a.wide ? launch_seg_kernel<L, SK, COLL, true, true, true>(a, nseg, rows, err, s)
                  : launch_seg_kernel<L, SK, COLL, true, false, true>(a, nseg, rows, err, s);
  if (a.wide)
    return fullbc ? launch_seg_kernel<L, SK, COLL, true, true, false>(a, nseg, rows, err, s)
                  : launch_seg_kernel<L, SK, COLL, false, true, false>(a, nseg, rows, err, s);
  return fullbc ? launch_seg_kernel<L, SK, COLL, true, false, false>(a, nseg, rows, err, s)
                : launch_seg_kernel<L, SK, COLL, false, false, false>(a, nseg, rows, err, s);
}

// Per-lattice entry (step_seg_*.cu): shifted FP16 / BF16 with collision code 3
// or 4; other combinations return -1.
template <int LAT>
int launch_seg_lattice(const StepArgs& a, int sk, int coll, bool fullbc, bool diag, int nseg, int rows, int* err,
                       cudaStream_t s) {
  if (sk == SK_F16S && coll == 3) return launch_seg_t<LAT, SK_F16S, 3>(a, fullbc, diag, nseg, rows, err, s);
  if (sk == SK_BF16S && coll == 3) return launch_seg_t<LAT, SK_BF16S, 3>(a, fullbc, diag, nseg, rows, err, s);
  if (sk == SK_F16S && coll == 4) return launch_seg_t<LAT, SK_F16S, 4>(a, fullbc, diag, nseg, rows, err, s);
  if (sk == SK_BF16S && coll == 4) return launch_seg_t<LAT, SK_BF16S, 4>(a, fullbc, diag, nseg, rows, err, s);
  return -1;
}

}  // namespace xlbg
