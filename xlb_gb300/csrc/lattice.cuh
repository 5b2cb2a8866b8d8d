// Compile-time lattice tables.
//
// Direction order is XLB's (xlb/velocity_set/d2q9.py:18-21, d3q19.py:19,
// d3q27.py:19): D3Q27 is itertools.product([0,-1,1], repeat=3) and D3Q19 keeps
// the entries with |c|_1 <= 2.  Weights follow d2q9.py:22, d3q19.py:20-27 and
// d3q27.py:20-29; opposite indices velocity_set.py:167-180; the packed second
// moment basis cc and the regularisation basis qi velocity_set.py:124-165.
//
// Every accessor is constexpr; the kernels call them inside fully unrolled
// loops so each lookup folds to an immediate.
#pragma once

namespace xlbg {

__host__ __device__ constexpr int tri_digit(int digit) { return digit == 0 ? 0 : (digit == 1 ? -1 : 1); }

// D3Q27 index l = 9a + 3b + e, component k takes digit (a, b, e)[k] mapped 0,1,2 -> 0,-1,1
__host__ __device__ constexpr int d3q27_c(int l, int k) {
  return tri_digit(k == 0 ? l / 9 : (k == 1 ? (l / 3) % 3 : l % 3));
}

// D3Q19 direction l is D3Q27 direction d3q19_map(l)
__host__ __device__ constexpr int d3q19_map(int l) {
  return l <= 12 ? l : (l == 13 ? 15 : (l == 14 ? 18 : (l == 15 ? 19 : (l == 16 ? 20 : (l == 17 ? 21 : 24)))));
}

__host__ __device__ constexpr int d2q9_c(int l, int k) {
  // cx = [0, 0, 0, 1, -1, 1, -1, 1, -1], cy = [0, 1, -1, 0, 1, -1, 0, 1, -1]
  return k == 0 ? ((l == 3 || l == 5 || l == 7) ? 1 : ((l == 4 || l == 6 || l == 8) ? -1 : 0))
                : ((l == 1 || l == 4 || l == 7) ? 1 : ((l == 2 || l == 5 || l == 8) ? -1 : 0));
}

template <int LAT>
struct Lattice;

// Opposite directions in closed form, so constant arguments fold to immediates.
// D3Q27: negate each base-3 digit (0 -> 0, 1 -> 2, 2 -> 1).
__host__ __device__ constexpr int d3q27_opp(int l) {
  return 9 * ((3 - l / 9) % 3) + 3 * ((3 - (l / 3) % 3) % 3) + (3 - l % 3) % 3;
}

template <>
struct Lattice<0> {  // D2Q9
  static constexpr int Q = 9, D = 2, NT = 3;
  __host__ __device__ static constexpr int c(int l, int k) { return d2q9_c(l, k); }
  // [0, 2, 1, 6, 5, 4, 3, 8, 7]
  __host__ __device__ static constexpr int opp(int l) {
    return l == 0 ? 0 : l == 1 ? 2 : l == 2 ? 1 : l == 3 ? 6 : l == 4 ? 5 : l == 5 ? 4 : l == 6 ? 3 : l == 7 ? 8 : 7;
  }
};

template <>
struct Lattice<1> {  // D3Q19
  static constexpr int Q = 19, D = 3, NT = 6;
  __host__ __device__ static constexpr int c(int l, int k) { return d3q27_c(d3q19_map(l), k); }
  // [0, 2, 1, 6, 8, 7, 3, 5, 4, 14, 16, 15, 18, 17, 9, 11, 10, 13, 12]
  __host__ __device__ static constexpr int opp(int l) {
    return l < 9 ? d3q27_opp(l)
                 : (l == 9 ? 14 : l == 10 ? 16 : l == 11 ? 15 : l == 12 ? 18 : l == 13 ? 17
                    : l == 14 ? 9 : l == 15 ? 11 : l == 16 ? 10 : l == 17 ? 13 : 12);
  }
};

template <>
struct Lattice<2> {  // D3Q27
  static constexpr int Q = 27, D = 3, NT = 6;
  __host__ __device__ static constexpr int c(int l, int k) { return d3q27_c(l, k); }
  __host__ __device__ static constexpr int opp(int l) { return d3q27_opp(l); }
};

template <class L>
__host__ __device__ constexpr int norm1(int l) {
  int s = 0;
  for (int k = 0; k < L::D; ++k) s += L::c(l, k) < 0 ? -L::c(l, k) : L::c(l, k);
  return s;
}

template <class L>
__host__ __device__ constexpr double weight(int l) {
  return L::Q == 9 ? (norm1<L>(l) == 0 ? 4.0 / 9.0 : (norm1<L>(l) == 1 ? 1.0 / 9.0 : 1.0 / 36.0))
         : L::Q == 19
             ? (norm1<L>(l) == 0 ? 1.0 / 3.0 : (norm1<L>(l) == 1 ? 1.0 / 18.0 : 1.0 / 36.0))
             : (norm1<L>(l) == 0 ? 8.0 / 27.0
                                 : (norm1<L>(l) == 1 ? 2.0 / 27.0 : (norm1<L>(l) == 2 ? 1.0 / 54.0 : 1.0 / 216.0)));
}

// Weight of the directions with |c|_1 = k (0 when the lattice has none).
template <class L>
__host__ __device__ constexpr double class_weight(int k) {
  for (int l = 0; l < L::Q; ++l)
    if (norm1<L>(l) == k) return weight<L>(l);
  return 0.0;
}

template <class L>
__host__ __device__ constexpr int opp(int l) {
  return L::opp(l);
}

// opp must send every direction to its negative (checked at compile time).
template <class L>
__host__ __device__ constexpr bool opp_is_negation() {
  for (int l = 0; l < L::Q; ++l)
    for (int k = 0; k < L::D; ++k)
      if (L::c(L::opp(l), k) != -L::c(l, k)) return false;
  return true;
}
static_assert(opp_is_negation<Lattice<0>>(), "D2Q9 opposite table");
static_assert(opp_is_negation<Lattice<1>>(), "D3Q19 opposite table");
static_assert(opp_is_negation<Lattice<2>>(), "D3Q27 opposite table");

// Packed symmetric-tensor component t -> axis pair (a, b), a <= b
template <class L>
__host__ __device__ constexpr int pair_a(int t) {
  return L::D == 2 ? (t == 2 ? 1 : 0) : (t < 3 ? 0 : (t < 5 ? 1 : 2));
}
template <class L>
__host__ __device__ constexpr int pair_b(int t) {
  return L::D == 2 ? (t == 0 ? 0 : 1) : (t == 0 ? 0 : (t == 1 ? 1 : (t == 2 ? 2 : (t == 3 ? 1 : (t == 4 ? 2 : 2)))));
}
template <class L>
__host__ __device__ constexpr int cc(int l, int t) {
  return L::c(l, pair_a<L>(t)) * L::c(l, pair_b<L>(t));
}
template <class L>
__host__ __device__ constexpr bool is_diag(int t) {
  return pair_a<L>(t) == pair_b<L>(t);
}
// qi = cc - 1/3 on the diagonal, 2 cc off the diagonal (computed in double, as XLB does)
template <class L>
__host__ __device__ constexpr double qi(int l, int t) {
  return is_diag<L>(t) ? (double)cc<L>(l, t) + (-1.0 / 3.0) : 2.0 * (double)cc<L>(l, t);
}

// Offset of direction l along internal axis k (0 slowest .. 2 fastest).  A 2D
// field (Q, nx, ny, 1) is the same memory as (Q, 1, nx, ny), so 2D lattices run
// on the internal grid (1, nx, ny) with c embedded as (0, cx, cy).
template <class L>
__host__ __device__ constexpr int axis_c(int l, int k) {
  return L::D == 3 ? L::c(l, k) : (k == 0 ? 0 : L::c(l, k - 1));
}

}  // namespace xlbg
