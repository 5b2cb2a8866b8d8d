// Store forms of the population fields.
//
// XLB casts to the compute type on load and to the store type on store
// (nse_stepper.py:309-310, :381, stream.py:80).  The shifted forms keep
// f - w_l in FP16 (scaled by 2^14) / BF16 and add w_l back on load; all conversions are the
// CUDA round-to-nearest-even intrinsics.  "raw" loads/stores are for boundary
// aux values, which are not populations and are never shifted.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace xlbg {

enum { SK_F32 = 0, SK_F64 = 1, SK_F16 = 2, SK_F16S = 3, SK_BF16S = 4 };

template <int SK, class T>
struct Store;

template <class T>
struct Store<SK_F32, T> {
  using S = float;
  using Bits = uint32_t;
  static constexpr bool shifted = false;
  __device__ static __forceinline__ T dec(Bits b, T) { return (T)__uint_as_float(b); }
  __device__ static __forceinline__ Bits enc(T v, T) { return __float_as_uint((float)v); }
  __device__ static __forceinline__ T dec_raw(Bits b) { return (T)__uint_as_float(b); }
  // deviation form (collision code 3, FP32 compute): g = f - w_l, exact for
  // w_l / 2 <= f <= 2 w_l (Sterbenz); the store rounds f = w_l + g once
  __device__ static __forceinline__ T dev(Bits b, T w) { return __uint_as_float(b) - w; }
  __device__ static __forceinline__ Bits enc_dev(T g, T w) { return __float_as_uint(g + w); }
};

template <class T>
struct Store<SK_F64, T> {
  using S = double;
  using Bits = unsigned long long;
  static constexpr bool shifted = false;
  __device__ static __forceinline__ T dec(Bits b, T) { return (T)__longlong_as_double((long long)b); }
  __device__ static __forceinline__ Bits enc(T v, T) { return (Bits)__double_as_longlong((double)v); }
  __device__ static __forceinline__ T dec_raw(Bits b) { return (T)__longlong_as_double((long long)b); }
};

__device__ __forceinline__ __half to_half(float v) { return __float2half_rn(v); }
__device__ __forceinline__ __half to_half(double v) { return __double2half(v); }

template <class T>
struct Store<SK_F16, T> {
  using S = __half;
  using Bits = unsigned short;
  static constexpr bool shifted = false;
  __device__ static __forceinline__ T dec(Bits b, T) { return (T)__half2float(__ushort_as_half(b)); }
  __device__ static __forceinline__ Bits enc(T v, T) { return __half_as_ushort(to_half(v)); }
  __device__ static __forceinline__ T dec_raw(Bits b) { return (T)__half2float(__ushort_as_half(b)); }
};

// FP16 holding (f - w_l) * 2^14.  The scale keeps deviations down to about 4e-9
// in FP16's normal range (smallest normal 6.1e-5); |f - w_l| < 4 fits.  Scaling
// by a power of two is exact, so each direction is one fused multiply-add whose
// result equals the separately rounded form (f - w_l) * 2^14 and h * 2^-14 + w_l
// bit for bit: fma(v, 2^14, -w 2^14) = RN(2^14 (v - w)) = 2^14 RN(v - w).
//
// The shifted forms also expose the stored deviation itself, g = kScale (f - w),
// for the collision evaluated on deviations (collision code 3): dev / enc_dev
// convert between the stored bits and g (one conversion each way; w unused).
template <>
struct Store<SK_F16S, float> {
  using S = __half;
  using Bits = unsigned short;
  static constexpr bool shifted = true;
  static constexpr float kScale = 16384.0f;
  static constexpr float kInvScale = 1.0f / 16384.0f;
  __device__ static __forceinline__ float dec(Bits b, float w) {
    return __fmaf_rn(__half2float(__ushort_as_half(b)), kInvScale, w);
  }
  __device__ static __forceinline__ Bits enc(float v, float w) {
    return __half_as_ushort(__float2half_rn(__fmaf_rn(v, kScale, -(w * kScale))));
  }
  __device__ static __forceinline__ float dec_raw(Bits b) { return __half2float(__ushort_as_half(b)); }
  __device__ static __forceinline__ float dev(Bits b, float) { return __half2float(__ushort_as_half(b)); }
  __device__ static __forceinline__ Bits enc_dev(float g, float) { return __half_as_ushort(__float2half_rn(g)); }
};

template <>
struct Store<SK_BF16S, float> {
  using S = __nv_bfloat16;
  using Bits = unsigned short;
  static constexpr bool shifted = true;
  static constexpr float kScale = 1.0f;
  static constexpr float kInvScale = 1.0f;
  __device__ static __forceinline__ float dec(Bits b, float w) {
    return __bfloat162float(__ushort_as_bfloat16(b)) + w;
  }
  __device__ static __forceinline__ Bits enc(float v, float w) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(v - w));
  }
  __device__ static __forceinline__ float dec_raw(Bits b) { return __bfloat162float(__ushort_as_bfloat16(b)); }
  __device__ static __forceinline__ float dev(Bits b, float) { return __bfloat162float(__ushort_as_bfloat16(b)); }
  __device__ static __forceinline__ Bits enc_dev(float g, float) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(g));
  }
};

// A pulled population as the collision code works on it: f for codes 0-2, the
// stored deviation g for code 3.
template <int SK, class T, int COLL>
__device__ __forceinline__ T load_pop(typename Store<SK, T>::Bits b, T w) {
  if constexpr (COLL >= 3)
    return Store<SK, T>::dev(b, w);
  else
    return Store<SK, T>::dec(b, w);
}

// The stored bits of a post-collision population (f for codes 0-2, g for codes
// 3 and 4; code 4 stores through sr_pack instead, in pairs).
template <int SK, class T, int COLL>
__device__ __forceinline__ typename Store<SK, T>::Bits store_pop(T v, T w) {
  if constexpr (COLL >= 3)
    return Store<SK, T>::enc_dev(v, w);
  else
    return Store<SK, T>::enc(v, w);
}

// Stochastic rounding of two FP32 values into a packed pair of the 16-bit store
// (collision code 4), Blackwell's cvt.rs: `hi` goes to the upper half with
// random bits rbits[31:16], `lo` to the lower half with rbits[15:0].  FP16: the
// result is floor(|x| / ulp + r13 / 2^13) ulp with r13 the low 13 of the 16 bits
// and ulp the FP16 ulp of |x|'s binade (2^-24 below 2^-14); +-inf from 65536 up.
// BF16: the 16 bits are added to the low half of x's FP32 pattern, which is then
// truncated.  (Both pinned bit for bit on 10^6 random pairs with random bits.)
template <int SK>
__device__ __forceinline__ uint32_t sr_pack(float lo, float hi, uint32_t rbits) {
  uint32_t d;
  if constexpr (SK == SK_F16S)
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  else
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}

// Random bits of one cell's stochastic rounding: C. Wellons' "lowbias32" integer
// hash of (cell, timestep), then one multiply by an odd constant per pair k of
// directions (the rounding needs bits independent of the values, uniform per
// value, fresh every step; runs stay reproducible).
__device__ __forceinline__ uint32_t sr_seed(uint32_t cell, uint32_t t) {
  uint32_t x = cell * 0x9E3779B1u + t * 0x85EBCA77u;
  x ^= x >> 16;
  x *= 0x7FEB352Du;
  x ^= x >> 15;
  x *= 0x846CA68Bu;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ uint32_t sr_bits(uint32_t seed, int k) {
  return seed * ((2u * (uint32_t)k + 1u) * 0x9E3779B9u);
}

template <class Bits>
__device__ __forceinline__ Bits ldg_bits(const Bits* p) {
  return __ldg(p);
}

}  // namespace xlbg
