// The fused time-step kernel: one thread per cell.
//
// Replaces XLB's Warp stepper kernel (xlb/operator/stepper/nse_stepper.py:344-382).
// Per cell, in XLB's order:
//   skip id 255 (:356-358) -> pull stream (stream.py:59-82) -> streaming-step BC
//   (:367) -> rho, u (:369) -> feq (:370) -> collision (:371) -> collision-step
//   BC and extrapolation aux data (:374, :286-293) -> store to f1 (:379-381).
// The aux recovery into f0 (:377) runs as a separate pass after this kernel
// (recovery.cuh), so that every pull of the step sees the unmodified f0.
//
// Memory traffic for a fluid cell is Q loads of f0 (the pull), one bc_mask byte
// and Q stores of f1.  missing_mask is read as one packed uint32, and f0/f1 own
// slots are read, only at boundary cells that need them.
//
// Grid: blockIdx.x = row (i0, i1) of the internal (n0, n1, n2) grid,
// blockIdx.y * blockDim.x + threadIdx.x = i2 along the contiguous axis, so each
// warp touches 32 consecutive cells of every population plane.
#pragma once
#include <stdint.h>

#include "lattice.cuh"
#include "physics.cuh"
#include "store.cuh"

namespace xlbg {

constexpr int kMaxBC = 16;
constexpr int kDiagSlots = 1024;
constexpr int kStepBlock = 256;

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
  long long ncell;
  int n0, n1, n2;
  int nbc;
  double omega;
  double extrap_cs;
  BCEntry bc[kMaxBC];
  int force_id;
  double* diag_slots;  // kDiagSlots x 4 doubles, zero on entry
};

__device__ __forceinline__ int wrap_dec(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrap_inc(int i, int n) { return i == n - 1 ? 0 : i + 1; }

template <class L, int SK, class T, int COLL, bool FULLBC, bool DIAG>
__global__ void __launch_bounds__(kStepBlock) step_kernel(const StepArgs a) {
  using St = Store<SK, T>;
  using Bits = typename St::Bits;
  constexpr int Q = L::Q;

  const Bits* __restrict__ f0 = static_cast<const Bits*>(a.f0);
  Bits* __restrict__ f1 = static_cast<Bits*>(a.f1);
  const long long N = a.ncell;
  const int n1 = a.n1, n2 = a.n2;

  const int row = blockIdx.x;
  const int i0 = row / n1;
  const int i1 = row - i0 * n1;
  const int i2 = blockIdx.y * kStepBlock + threadIdx.x;
  const bool inside = i2 < n2;
  const long long cell = (long long)row * n2 + i2;

  double dmass = 0.0, dforce[3] = {0.0, 0.0, 0.0};

  const uint8_t id = inside ? a.bc_mask[cell] : (uint8_t)255;
  if (id != 255) {
    // ---- pull stream ----
    T f[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      const int s0 = axis_c<L>(l, 0) == 1 ? wrap_dec(i0, a.n0) : (axis_c<L>(l, 0) == -1 ? wrap_inc(i0, a.n0) : i0);
      const int s1 = axis_c<L>(l, 1) == 1 ? wrap_dec(i1, n1) : (axis_c<L>(l, 1) == -1 ? wrap_inc(i1, n1) : i1);
      const int s2 = axis_c<L>(l, 2) == 1 ? wrap_dec(i2, n2) : (axis_c<L>(l, 2) == -1 ? wrap_inc(i2, n2) : i2);
      const long long src = ((long long)s0 * n1 + s1) * n2 + s2;
      f[l] = St::dec(ldg_bits(f0 + (long long)l * N + src), T(weight<L>(l)));
    }

    // ---- boundary lookup (XLB unrolls the BC list the same way, nse_stepper.py:280-293) ----
    int kind = 0;
    double bc_rho = 0.0, bc_u[3] = {0.0, 0.0, 0.0};
    uint32_t miss = 0;
    if (id != 0) {
#pragma unroll
      for (int b = 0; b < kMaxBC; ++b) {
        if (b < a.nbc && a.bc[b].id == (int)id) {
          kind = a.bc[b].kind;
          bc_rho = a.bc[b].rho;
          bc_u[0] = a.bc[b].u[0];
          bc_u[1] = a.bc[b].u[1];
          bc_u[2] = a.bc[b].u[2];
        }
      }
      const bool need_miss = kind == BC_HALFWAY || kind == BC_EXTRAP || kind == BC_ZOUHE_V || kind == BC_ZOUHE_P ||
                             kind == BC_REG_V || kind == BC_REG_P || (DIAG && (int)id == a.force_id);
      if (need_miss) miss = __ldg(a.miss + cell);

      // ---- streaming-step BCs: f_pre = own-cell f0, f_post = pulled values ----
      if (kind == BC_HALFWAY || (FULLBC && kind == BC_EXTRAP)) {
        // bc_halfway_bounce_back.py:163-171, bc_extrapolation_outflow.py:383-388
#pragma unroll
        for (int l = 0; l < Q; ++l) {
          if ((miss >> l) & 1u)
            f[l] = St::dec(ldg_bits(f0 + (long long)opp<L>(l) * N + cell), T(weight<L>(opp<L>(l))));
        }
      } else if (kind == BC_EQUILIBRIUM) {
        // bc_equilibrium.py:255-271
        T u[L::D];
#pragma unroll
        for (int d = 0; d < L::D; ++d) u[d] = T(bc_u[d]);
        equilibrium<L>(T(bc_rho), u, f);
      } else if (FULLBC && kind >= BC_ZOUHE_V && kind <= BC_REG_P) {
        // the prescribed value lives in slot 0 of f1 (boundary_condition.py:151-152)
        const T aux = St::dec_raw(ldg_bits(f1 + cell));
        zouhe_like<L>(f, miss, aux, kind);
      }
    }

    // ---- macroscopic, equilibrium, collision ----
    T rho, u[L::D];
    macroscopic<L>(f, rho, u);
    T feq[Q];
    equilibrium<L>(rho, u, feq);
    const T omega = T(a.omega);
    T fo[Q];
    if constexpr (COLL == 0) {
#pragma unroll
      for (int l = 0; l < Q; ++l) fo[l] = f[l] - omega * (f[l] - feq[l]);
    } else {
      kbc<L>(f, feq, rho, omega, fo);
    }

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
      const int ii[3] = {i0, i1, i2};
      const int nn[3] = {a.n0, n1, n2};
#pragma unroll
      for (int l = 0; l < Q; ++l) {
        if ((miss >> l) & 1u) {
          int s[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const int off = axis_c<L>(l, k) + (L::D == 3 ? nv[k] : (k == 0 ? 0 : nv[k - 1]));
            int v = (ii[k] - off) % nn[k];
            s[k] = v < 0 ? v + nn[k] : v;
          }
          const long long src = ((long long)s[0] * n1 + s[1]) * n2 + s[2];
          const T faux = St::dec(ldg_bits(f0 + (long long)l * N + src), T(weight<L>(l)));
          fo[opp<L>(l)] = (T(1) - cs) * f[l] + cs * faux;
        }
      }
    }

    // ---- store ----
    T msum = T(0);
#pragma unroll
    for (int l = 0; l < Q; ++l) {
      const Bits b = St::enc(fo[l], T(weight<L>(l)));
      f1[(long long)l * N + cell] = b;
      if constexpr (DIAG) {
        // mass of the stored state, summed per cell in T
        const T v = St::dec(b, T(weight<L>(l)));
        msum = l == 0 ? v : msum + v;
      }
    }
    if constexpr (DIAG) {
      dmass = (double)msum;
      if ((int)id == a.force_id && !(miss & 1u)) {
        // momentum exchange on the input state (momentum_transfer.py:130-158):
        // phi_l = f0[opp l] + f_post_stream[l] with f_post_stream[l] = f0[opp l]
        T m[L::D];
#pragma unroll
        for (int d = 0; d < L::D; ++d) m[d] = T(0);
#pragma unroll
        for (int l = 0; l < Q; ++l) {
          if ((miss >> l) & 1u) {
            const T v = St::dec(ldg_bits(f0 + (long long)opp<L>(l) * N + cell), T(weight<L>(opp<L>(l))));
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

  if constexpr (DIAG) {
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
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        double x = lane < kStepBlock / 32 ? red[lane][k] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) {
          const unsigned slot = (blockIdx.x * gridDim.y + blockIdx.y) % kDiagSlots;
          atomicAdd(a.diag_slots + slot * 4 + k, x);
        }
      }
    }
  }
}

}  // namespace xlbg
