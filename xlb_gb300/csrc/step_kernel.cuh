// The fused time-step kernels.
//
// Replaces XLB's Warp stepper kernel (xlb/operator/stepper/nse_stepper.py:344-382).
// Per cell, in XLB's order:
//   skip id 255 (:356-358) -> pull stream (stream.py:59-82) -> streaming-step BC
//   (:367) -> rho, u (:369) -> feq (:370) -> collision (:371) -> collision-step
//   BC and extrapolation aux data (:374, :286-293) -> store to f1 (:379-381).
// The aux recovery into f0 (:377) runs as separate passes around this kernel
// (recovery_save / recovery_restore in api.cu), so that every pull of the step
// sees the unmodified f0.
//
// Memory traffic for a fluid cell is Q loads of f0 (the pull), one bc_mask byte
// and Q stores of f1.  missing_mask is read as one packed uint32, and f0/f1 own
// slots are read, only at boundary cells that need them.
//
// Grid: blockIdx.x = row (i0, i1) of the internal (n0, n1, n2) grid; threads
// run along the contiguous axis i2 (one cell per thread in step_kernel, V cells
// per thread in step_kernel_vec), so each warp touches consecutive cells of
// every population plane.
#pragma once
#include <stdint.h>

#include "lattice.cuh"
#include "physics.cuh"
#include "store.cuh"

namespace xlbg {

constexpr int kMaxBC = 16;
constexpr int kDiagSlots = 1024;
constexpr int kStepBlock = 256;  // upper bound on threads per block

struct BCEntry {
  int id;
  int kind;
  double rho;
  double u[3];
};

struct StepArgs {
  const void* f0;
  void* f1;
  const uint8_t* bc_mask;
  const uint32_t* miss;
  // one store-type value per cell holding the ZouHe / Regularized prescribed
  // values: plane 0 of f1 in XLB's encoding (boundary_condition.py:151-152),
  // or a separate field for the recording and adjoint entry points
  const void* aux;
  long long ncell;
  int wide;  // Q * ncell >= 2^32: the marching kernel indexes planes in 64 bits
  int n0, n1, n2;
  int nbc;
  double omega;
  float omega_f;  // omega rounded to float on the host (same RN conversion as in-kernel)
  double extrap_cs;
  BCEntry bc[kMaxBC];
  // per bc_mask id: kind | (index into bc) << 8; 0 for ids without a BC.  One
  // constant load per boundary cell instead of a scan over the BC list.
  uint16_t bc_code[256];
  int force_id;
  double* diag_slots;  // kDiagSlots x 4 doubles, zero on entry
  unsigned timestep;   // the step's timestep argument (seeds the stochastic rounding of code 4)
};

// Element (l, i) of f0 / f1 in the store type.  Idx is the index type of the
// whole plane-and-cell offset: long long in general, unsigned 32-bit in the
// marching kernel, which runs only when Q * cells < 2^32 (the host checks) and
// saves the 64-bit multiply per access.
template <class Bits, class Idx>
__device__ __forceinline__ const Bits* at0(const StepArgs& a, int l, Idx i) {
  return static_cast<const Bits*>(a.f0) + ((Idx)l * (Idx)a.ncell + i);
}
template <class Bits, class Idx>
__device__ __forceinline__ Bits* at1(const StepArgs& a, int l, Idx i) {
  return static_cast<Bits*>(a.f1) + ((Idx)l * (Idx)a.ncell + i);
}

template <class T>
__device__ __forceinline__ T omega_of(const StepArgs& a) {
  if constexpr (sizeof(T) == 4)
    return a.omega_f;
  else
    return T(a.omega);
}

// Offset of the source row (i0 - c0, i1 - c1), with the one-cell wrap, for a
// direction's (c0, c1); block-uniform.
template <int C0, int C1>
__device__ __forceinline__ long long row_offset(int i0, int i1, int n0, int n1, int n2) {
  const int s0 = C0 == 1 ? (i0 == 0 ? n0 - 1 : i0 - 1) : (C0 == -1 ? (i0 == n0 - 1 ? 0 : i0 + 1) : i0);
  const int s1 = C1 == 1 ? (i1 == 0 ? n1 - 1 : i1 - 1) : (C1 == -1 ? (i1 == n1 - 1 ? 0 : i1 + 1) : i1);
  return ((long long)s0 * n1 + s1) * n2;
}

// The nine neighbour-row offsets (c0, c1) in {1, 0, -1}^2, index (c0 + 1) * 3 + (c1 + 1).
struct RowOffsets {
  long long r[9];
  __device__ __forceinline__ RowOffsets(int i0, int i1, int n0, int n1, int n2) {
    r[0] = row_offset<-1, -1>(i0, i1, n0, n1, n2);
    r[1] = row_offset<-1, 0>(i0, i1, n0, n1, n2);
    r[2] = row_offset<-1, 1>(i0, i1, n0, n1, n2);
    r[3] = row_offset<0, -1>(i0, i1, n0, n1, n2);
    r[4] = row_offset<0, 0>(i0, i1, n0, n1, n2);
    r[5] = row_offset<0, 1>(i0, i1, n0, n1, n2);
    r[6] = row_offset<1, -1>(i0, i1, n0, n1, n2);
    r[7] = row_offset<1, 0>(i0, i1, n0, n1, n2);
    r[8] = row_offset<1, 1>(i0, i1, n0, n1, n2);
  }
  template <class L>
  __device__ __forceinline__ long long of(int l) const {
    return r[(axis_c<L>(l, 0) + 1) * 3 + (axis_c<L>(l, 1) + 1)];
  }
};

__device__ __forceinline__ int wrap_dec(int i, int n) { return i == 0 ? n - 1 : i - 1; }
// periodic wrap of an index at most one period outside [0, n)
__device__ __forceinline__ int wrap_any(int v, int n) {
  v = v < 0 ? v + n : v;
  return v >= n ? v - n : v;
}
__device__ __forceinline__ int wrap_inc(int i, int n) { return i == n - 1 ? 0 : i + 1; }

// Pull stream for one cell: f[l] = f0[l, x - c_l] with XLB's one-cell periodic
// wrap (stream.py:64-82).
// With collision code 3 the values are the stored deviations (load_pop).
template <class L, int SK, class T, int COLL>
__device__ __forceinline__ void pull_cell(const StepArgs& a, int i0, int i1, int i2, T (&f)[L::Q]) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  const int n2 = a.n2;
  const RowOffsets rows(i0, i1, a.n0, a.n1, n2);
  const int z[3] = {i2 == n2 - 1 ? 0 : i2 + 1, i2, i2 == 0 ? n2 - 1 : i2 - 1};  // source i2 for c2 = -1, 0, +1
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    f[l] = load_pop<SK, T, COLL>(ldg_bits(at0<Bits>(a, l, rows.of<L>(l) + z[axis_c<L>(l, 2) + 1])), T(weight<L>(l)));
  }
}

// Collision of one cell: XLB-order BGK (COLL 0), KBC (COLL 1), pair-form BGK
// (COLL 2) or BGK on deviations (COLL 3; COLL 4 the same with stochastic rounding
// of the stores).
template <class L, int SK, class T, int COLL>
__device__ __forceinline__ void collide(const T (&f)[L::Q], T omega, T (&fo)[L::Q]) {
  if constexpr (COLL >= 3) {
    bgk_shifted<L, SK>(f, omega, fo);
  } else if constexpr (COLL == 2) {
    bgk_pair<L>(f, omega, fo);
  } else {
    T rho, u[L::D];
    macroscopic<L>(f, rho, u);
    T feq[L::Q];
    equilibrium<L>(rho, u, feq);
    if constexpr (COLL == 0) {
#pragma unroll
      for (int l = 0; l < L::Q; ++l) fo[l] = f[l] - omega * (f[l] - feq[l]);
    } else {
      kbc<L>(f, feq, rho, omega, fo);
    }
  }
}

// Store of one cell's post-collision populations (nse_stepper.py:379-381); with
// DIAG, the cell's mass as stored, summed in T.
template <class L, int SK, class T, int COLL, bool DIAG, class Idx>
__device__ __forceinline__ void store_cell(const StepArgs& a, Idx cell, const T (&fo)[L::Q], double& dmass) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  T msum = T(0);
  // 16-bit stores address the cell's slot in plane 0 plus launch-uniform plane
  // offsets (measured 3 % faster for them); 32/64-bit stores keep one 32-bit
  // plane-and-cell offset per store (3 % faster for FP32)
  Bits* __restrict__ row1 = static_cast<Bits*>(a.f1) + cell;
  const size_t plane = (size_t)a.ncell;
  if constexpr (COLL == 4) {
    // stochastic rounding, directions in pairs (the last one alone when Q is odd)
    const uint32_t seed = sr_seed((uint32_t)cell, a.timestep);
#pragma unroll
    for (int l = 0; l < L::Q; l += 2) {
      const uint32_t p = sr_pack<SK>(fo[l], l + 1 < L::Q ? fo[l + 1] : 0.0f, sr_bits(seed, l / 2));
      row1[(size_t)l * plane] = (Bits)(p & 0xffffu);
      if (l + 1 < L::Q) row1[(size_t)(l + 1) * plane] = (Bits)(p >> 16);
      if constexpr (DIAG) {
        const T v = St::dec((Bits)(p & 0xffffu), T(weight<L>(l)));
        msum = l == 0 ? v : msum + v;
        if (l + 1 < L::Q) msum = msum + St::dec((Bits)(p >> 16), T(weight<L>(l + 1)));
      }
    }
    if constexpr (DIAG) dmass = (double)msum;
    return;
  }
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    const Bits b = store_pop<SK, T, COLL>(fo[l], T(weight<L>(l)));
    if constexpr (sizeof(Bits) == 2)
      row1[(size_t)l * plane] = b;
    else
      *at1<Bits>(a, l, cell) = b;
    if constexpr (DIAG) {
      const T v = St::dec(b, T(weight<L>(l)));
      msum = l == 0 ? v : msum + v;
    }
  }
  if constexpr (DIAG) dmass = (double)msum;
}

// The same store for a cell index below 2^31 (the TMA-staged kernel's fluid
// path): each direction's plane base is launch-uniform and the cell index 32-bit,
// so an address is one wide multiply-add of the cell index onto the plane base
// rather than a 64-bit add to a per-cell pointer.
template <class L, int SK, class T, int COLL, bool DIAG>
__device__ __forceinline__ void store_cell_u32(const StepArgs& a, unsigned cell, const T (&fo)[L::Q],
                                               double& dmass) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  T msum = T(0);
  const size_t plane = (size_t)a.ncell;
  if constexpr (COLL == 4) {
    const uint32_t seed = sr_seed(cell, a.timestep);
#pragma unroll
    for (int l = 0; l < L::Q; l += 2) {
      const uint32_t p = sr_pack<SK>(fo[l], l + 1 < L::Q ? fo[l + 1] : 0.0f, sr_bits(seed, l / 2));
      (static_cast<Bits*>(a.f1) + (size_t)l * plane)[cell] = (Bits)(p & 0xffffu);
      if (l + 1 < L::Q) (static_cast<Bits*>(a.f1) + (size_t)(l + 1) * plane)[cell] = (Bits)(p >> 16);
      if constexpr (DIAG) {
        const T v = St::dec((Bits)(p & 0xffffu), T(weight<L>(l)));
        msum = l == 0 ? v : msum + v;
        if (l + 1 < L::Q) msum = msum + St::dec((Bits)(p >> 16), T(weight<L>(l + 1)));
      }
    }
    if constexpr (DIAG) dmass = (double)msum;
    return;
  }
#pragma unroll
  for (int l = 0; l < L::Q; ++l) {
    const Bits b = store_pop<SK, T, COLL>(fo[l], T(weight<L>(l)));
    Bits* __restrict__ base = static_cast<Bits*>(a.f1) + (size_t)l * plane;
    base[cell] = b;
    if constexpr (DIAG) {
      const T v = St::dec(b, T(weight<L>(l)));
      msum = l == 0 ? v : msum + v;
    }
  }
  if constexpr (DIAG) dmass = (double)msum;
}

// Everything after the pull for one cell: BC lookup, streaming-step BC,
// collision, collision-step BC, store to f1 and the diagnostics contributions.
// f holds the pulled values of the cell; the cell is not a skip cell (id 255).
// With collision code 3 every value in f and fo is a deviation g: the
// bounce-back kinds copy deviations (w_l = w_opp l), the extrapolation blend is
// linear, and EquilibriumBC / ZouHe / Regularized run on deviations too
// (equilibrium_dev, zouhe_like_dev).
// The collision is inlined once, shared by fluid and boundary cells (a second
// copy for a fluid-only path doubled the code and ran slower).
template <class L, int SK, class T, int COLL, bool FULLBC, bool DIAG, class Idx>
__device__ __forceinline__ void cell_update(const StepArgs& a, int i0, int i1, int i2, Idx cell, uint8_t id,
                                            T (&f)[L::Q], double& dmass, double (&dforce)[3]) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;
  const int n1 = a.n1, n2 = a.n2;
  // ---- boundary lookup (XLB unrolls the BC list, nse_stepper.py:280-293; here
  // one table load gives the kind and the BC's slot) ----
  int kind = 0;
  uint32_t miss = 0;
  if (id != 0) {
    const unsigned code = a.bc_code[id];
    kind = (int)(code & 0xffu);
    const int slot = (int)(code >> 8);
    const bool need_miss = kind == BC_HALFWAY || kind == BC_EXTRAP || kind == BC_ZOUHE_V || kind == BC_ZOUHE_P ||
                           kind == BC_REG_V || kind == BC_REG_P || (DIAG && (int)id == a.force_id);
    if (need_miss) miss = __ldg(a.miss + cell);

    // ---- streaming-step BCs: f_pre = own-cell f0, f_post = pulled values ----
    if (kind == BC_HALFWAY || (FULLBC && kind == BC_EXTRAP)) {
      // bc_halfway_bounce_back.py:163-171, bc_extrapolation_outflow.py:383-388
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        if ((miss >> l) & 1u)
          f[l] = load_pop<SK, T, COLL>(ldg_bits(at0<Bits>(a, opp<L>(l), cell)), T(weight<L>(opp<L>(l))));
      }
    } else if (kind == BC_EQUILIBRIUM) {
      // bc_equilibrium.py:255-271
      T u[L::D];
#pragma unroll
      for (int d = 0; d < L::D; ++d) u[d] = T(a.bc[slot].u[d]);
      if constexpr (COLL >= 3)
        equilibrium_dev<L, SK>((float)(a.bc[slot].rho - 1.0), u, f);
      else
        equilibrium<L>(T(a.bc[slot].rho), u, f);
    } else if (FULLBC && kind >= BC_ZOUHE_V && kind <= BC_REG_P) {
      // the prescribed value lives in slot 0 of f1 (boundary_condition.py:151-152)
      const T aux = St::dec_raw(static_cast<const Bits*>(a.aux)[cell]);
      if constexpr (COLL >= 3)
        zouhe_like_dev<L, SK>(f, miss, aux, kind);
      else
        zouhe_like<L>(f, miss, aux, kind);
    }
  }

  // ---- macroscopic, equilibrium, collision ----
  T fo[Q];
  collide<L, SK, T, COLL>(f, omega_of<T>(a), fo);

  // ---- collision-step BCs ----
  if (kind == BC_FULLWAY) {
    // bc_fullway_bounce_back.py:59-72
#pragma unroll
    for (int l = 0; l < Q; ++l) fo[l] = f[opp<L>(l)];
  } else if (FULLBC && kind == BC_EXTRAP) {
    // bc_extrapolation_outflow.py:390-415: store extrapolated values in the
    // outgoing slots; the neighbour read wraps like the stream does.
    int nv[L::D];
    normal_of<L>(miss, nv);
    const T cs = T(a.extrap_cs);
    // the normal on the internal axes (2D embeds as (0, nx, ny))
    const int m0 = L::D == 3 ? nv[0] : 0;
    const int m1 = L::D == 3 ? nv[1] : nv[0];
    const int m2 = L::D == 3 ? nv[2] : nv[1];
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      if ((miss >> l) & 1u) {
        const int s0 = wrap_any(i0 - (axis_c<L>(l, 0) + m0), a.n0);
        const int s1 = wrap_any(i1 - (axis_c<L>(l, 1) + m1), n1);
        const int s2 = wrap_any(i2 - (axis_c<L>(l, 2) + m2), n2);
        const long long src = ((long long)s0 * n1 + s1) * n2 + s2;
        const T faux = load_pop<SK, T, COLL>(ldg_bits(at0<Bits>(a, l, (Idx)src)), T(weight<L>(l)));
        fo[opp<L>(l)] = (T(1) - cs) * f[l] + cs * faux;
      }
    }
  }

  store_cell<L, SK, T, COLL, DIAG>(a, cell, fo, dmass);
  if constexpr (DIAG) {
    if ((int)id == a.force_id && !(miss & 1u)) {
      // momentum exchange on the input state (momentum_transfer.py:130-158):
      // phi_l = f0[opp l] + f_post_stream[l] with f_post_stream[l] = f0[opp l]
      T m[L::D];
#pragma unroll
      for (int d = 0; d < L::D; ++d) m[d] = T(0);
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        if ((miss >> l) & 1u) {
          const T v = St::dec(ldg_bits(at0<Bits>(a, opp<L>(l), cell)), T(weight<L>(opp<L>(l))));
          const T phi = v + v;
#pragma unroll
          for (int d = 0; d < L::D; ++d) {
            if (L::c(opp<L>(l), d) == 1) m[d] = m[d] + phi;
            if (L::c(opp<L>(l), d) == -1) m[d] = m[d] - phi;
          }
        }
      }
#pragma unroll
      for (int d = 0; d < L::D; ++d) dforce[d] = (double)m[d];
    }
  }
}

// Block reduction of the four FP64 diagnostics into the slot array.
__device__ __forceinline__ void reduce_diag(double dmass, const double (&dforce)[3], double* slots) {
  __shared__ double red[kStepBlock / 32][4];
  double v[4] = {dmass, dforce[0], dforce[1], dforce[2]};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) red[warp][k] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double x = lane < nw ? red[lane][k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) {
        const unsigned slot = (blockIdx.x * gridDim.y + blockIdx.y) % kDiagSlots;
        atomicAdd(slots + slot * 4 + k, x);
      }
    }
  }
}

// One cell per thread.
template <class L, int SK, class T, int COLL, bool FULLBC, bool DIAG>
__global__ void __launch_bounds__(kStepBlock) step_kernel(const StepArgs a) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;

  const int n1 = a.n1, n2 = a.n2;

  const int row = blockIdx.x;
  const int i0 = row / n1;
  const int i1 = row - i0 * n1;
  const int i2 = blockIdx.y * blockDim.x + threadIdx.x;
  const bool inside = i2 < n2;
  const long long cell = (long long)row * n2 + i2;

  double dmass = 0.0, dforce[3] = {0.0, 0.0, 0.0};

  const uint8_t id = inside ? a.bc_mask[cell] : (uint8_t)255;
  if (id != 255) {
    T f[Q];
    pull_cell<L, SK, T, COLL>(a, i0, i1, i2, f);
    cell_update<L, SK, T, COLL, FULLBC, DIAG>(a, i0, i1, i2, cell, id, f, dmass, dforce);
  }
  if constexpr (DIAG) reduce_diag(dmass, dforce, a.diag_slots);
}

// ---------------------------------------------------------------------------
// Marching kernel: each thread owns one position i2 on the contiguous axis and
// one position i0 on axis 0, and walks a chunk of rows i1 = r0 .. r0+CH-1.
// Set-up (axis-0 plane offsets and contiguous-axis wraps, all with XLB's
// one-cell periodic wrap) is done once per thread; per cell only the three
// block-uniform row offsets of axis 1 change.  2D lattices have n0 = 1 and
// march along x.  Arithmetic per cell is cell_update's, unchanged.
// Grid: blockIdx.x = i0 * ceil(n2 / blockDim.x) + i2 chunk, blockIdx.y = row chunk.
// ---------------------------------------------------------------------------
// Resident blocks per SM asked of the register allocator: with FP32 compute, four
// 256-thread blocks (at most 64 registers a thread) for D2Q9 and D3Q19, where the
// step is bound by memory parallelism, and two for D3Q27, whose 27 populations
// need more registers; FP64 compute keeps the allocator's choice.
template <class L, class T>
constexpr int march_min_blocks() {
  return sizeof(T) != 4 ? 1 : (L::Q <= 19 ? 4 : 2);
}

// Idx: type of the plane-and-cell offsets, unsigned when Q * cells < 2^32, else
// long long (cell offsets stay 32-bit: the host runs this kernel for < 2^31 cells).
// DIAG: the diagnostics step (mass of the output, force on the input; see
// cell_update) -- per-thread FP64 sums over the rows it walks, then the block
// reduction into the slot array.  Threads past the contiguous axis then stay to
// the end for the reduction's barrier.
template <class L, int SK, class T, int COLL, bool FULLBC, class Idx, bool DIAG = false>
__global__ void __launch_bounds__(kStepBlock, march_min_blocks<L, T>()) step_kernel_march(const StepArgs a, int chunk) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;

  const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
  const int zblocks = (n2 + blockDim.x - 1) / blockDim.x;
  const int i0 = blockIdx.x / zblocks;
  const int i2 = (blockIdx.x - i0 * zblocks) * blockDim.x + threadIdx.x;
  if constexpr (!DIAG) {
    if (i2 >= n2) return;
  }
  const bool inside = i2 < n2;
  const unsigned plane = (unsigned)n1 * (unsigned)n2;
  // source index parts along axes 0 and 2 for c = -1, 0, +1 (index c + 1)
  const unsigned xo[3] = {(unsigned)(i0 == n0 - 1 ? 0 : i0 + 1) * plane, (unsigned)i0 * plane,
                          (unsigned)(i0 == 0 ? n0 - 1 : i0 - 1) * plane};
  const unsigned zo[3] = {(unsigned)(i2 == n2 - 1 ? 0 : i2 + 1), (unsigned)i2, (unsigned)(i2 == 0 ? n2 - 1 : i2 - 1)};
  unsigned xz[3][3];
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q) xz[p][q] = xo[p] + zo[q];
  const int r0 = blockIdx.y * chunk;
  const int r1 = !inside ? r0 : (r0 + chunk < n1 ? r0 + chunk : n1);
  double dm = 0.0, df[3] = {0.0, 0.0, 0.0};
  for (int i1 = r0; i1 < r1; ++i1) {
    const unsigned yo[3] = {(unsigned)(i1 == n1 - 1 ? 0 : i1 + 1) * (unsigned)n2, (unsigned)i1 * (unsigned)n2,
                            (unsigned)(i1 == 0 ? n1 - 1 : i1 - 1) * (unsigned)n2};
    const unsigned cell = xz[1][1] + yo[1];
    const uint8_t id = a.bc_mask[cell];
    if (id == 255) continue;
    T f[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      const unsigned src = xz[axis_c<L>(l, 0) + 1][axis_c<L>(l, 2) + 1] + yo[axis_c<L>(l, 1) + 1];
      f[l] = load_pop<SK, T, COLL>(ldg_bits(at0<Bits>(a, l, (Idx)src)), T(weight<L>(l)));
    }
    if constexpr (DIAG) {
      double dmc = 0.0, dfc[3] = {0.0, 0.0, 0.0};
      cell_update<L, SK, T, COLL, FULLBC, true>(a, i0, i1, i2, (Idx)cell, id, f, dmc, dfc);
      dm += dmc;
      df[0] += dfc[0];
      df[1] += dfc[1];
      df[2] += dfc[2];
    } else {
      cell_update<L, SK, T, COLL, FULLBC, false>(a, i0, i1, i2, (Idx)cell, id, f, dm, df);
    }
  }
  if constexpr (DIAG) reduce_diag(dm, df, a.diag_slots);
}

}  // namespace xlbg
