// C ABI of libxlbg.so (declarations and per-entry documentation in include/xlbg.h),
// plus the small set-up kernels: missing-mask packing, equilibrium fill,
// macroscopic read-out, aux-recovery passes and the diagnostics finaliser.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>
#include <cmath>
#include <string>

#include "../../include/xlbg.h"
#include "step_dispatch.cuh"

namespace xlbg {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

static int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return XLBG_OK;
  return fail(XLBG_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

int store_bytes(int sk) { return sk == SK_F64 ? 8 : (sk == SK_F32 ? 4 : 2); }

static int lattice_q(int lat) { return lat == 0 ? 9 : (lat == 1 ? 19 : 27); }
static int lattice_d(int lat) { return lat == 0 ? 2 : 3; }

static bool needs_full_bc(const xlbg_desc* d) {
  for (int b = 0; b < d->nbc; ++b) {
    const int k = d->bc[b].kind;
    if (k == XLBG_BC_ZOUHE_VELOCITY || k == XLBG_BC_ZOUHE_PRESSURE || k == XLBG_BC_REGULARIZED_VELOCITY ||
        k == XLBG_BC_REGULARIZED_PRESSURE || k == XLBG_BC_EXTRAPOLATION)
      return true;
  }
  return false;
}

static int check_desc(const xlbg_desc* d) {
  if (!d) return fail(XLBG_ERR_ARG, "desc is NULL");
  if (d->abi_version != XLBG_ABI_VERSION)
    return fail(XLBG_ERR_ARG, "desc abi_version %d, library %d", d->abi_version, XLBG_ABI_VERSION);
  if (d->lattice < 0 || d->lattice > 2) return fail(XLBG_ERR_ARG, "unknown lattice %d", d->lattice);
  if (d->store < 0 || d->store > 4) return fail(XLBG_ERR_ARG, "unknown store form %d", d->store);
  if (d->compute != XLBG_COMPUTE_F32 && d->compute != XLBG_COMPUTE_F64)
    return fail(XLBG_ERR_ARG, "unknown compute type %d", d->compute);
  if (d->compute == XLBG_COMPUTE_F64 && (d->store == XLBG_STORE_F16S || d->store == XLBG_STORE_BF16S))
    return fail(XLBG_ERR_UNSUPPORTED, "shifted FP16/BF16 storage is defined with FP32 compute only");
  if (d->collision != XLBG_BGK && d->collision != XLBG_KBC && d->collision != XLBG_BGK_PAIR &&
      d->collision != XLBG_BGK_SHIFTED && d->collision != XLBG_BGK_SHIFTED_SR)
    return fail(XLBG_ERR_ARG, "unknown collision %d", d->collision);
  if (d->collision == XLBG_BGK_SHIFTED_SR &&
      !(d->compute == XLBG_COMPUTE_F32 && (d->store == XLBG_STORE_F16S || d->store == XLBG_STORE_BF16S)))
    return fail(XLBG_ERR_UNSUPPORTED, "stochastic rounding needs FP32 compute with a shifted FP16/BF16 store");
  if (d->collision == XLBG_BGK_SHIFTED &&
      !(d->compute == XLBG_COMPUTE_F32 &&
        (d->store == XLBG_STORE_F16S || d->store == XLBG_STORE_BF16S || d->store == XLBG_STORE_F32)))
    return fail(XLBG_ERR_UNSUPPORTED, "BGK on deviations needs FP32 compute with an FP32 or shifted FP16/BF16 store");
  if (d->collision == XLBG_KBC && d->lattice == XLBG_D3Q19)
    return fail(XLBG_ERR_UNSUPPORTED, "KBC collision is defined for D2Q9 and D3Q27 only (kbc.py:184-185)");
  if (d->nx <= 0 || d->ny <= 0 || d->nz <= 0) return fail(XLBG_ERR_ARG, "grid shape must be positive");
  if (d->lattice == XLBG_D2Q9 && d->nz != 1) return fail(XLBG_ERR_ARG, "2D grids have nz == 1");
  const long long rows = d->lattice == XLBG_D2Q9 ? d->nx : d->nx * d->ny;
  const long long fast = d->lattice == XLBG_D2Q9 ? d->ny : d->nz;
  if (rows > 0x7fffffffLL || fast > 0x7fffffffLL || d->nx > 0x7fffffffLL || d->ny > 0x7fffffffLL)
    return fail(XLBG_ERR_ARG, "grid too large");
  if (d->nbc < 0 || d->nbc > XLBG_MAX_BC) return fail(XLBG_ERR_ARG, "nbc %d outside 0..%d", d->nbc, XLBG_MAX_BC);
  for (int b = 0; b < d->nbc; ++b) {
    if (d->bc[b].id < 1 || d->bc[b].id > 254) return fail(XLBG_ERR_ARG, "bc id %d outside 1..254", d->bc[b].id);
    if (d->bc[b].kind < XLBG_BC_FULLWAY_BB || d->bc[b].kind > XLBG_BC_EXTRAPOLATION)
      return fail(XLBG_ERR_ARG, "bc kind %d unknown", d->bc[b].kind);
    for (int c = 0; c < b; ++c)
      if (d->bc[c].id == d->bc[b].id) return fail(XLBG_ERR_ARG, "bc id %d listed twice", d->bc[b].id);
  }
  return XLBG_OK;
}

int check_desc_public(const xlbg_desc* d) { return check_desc(d); }

int check_ptr(const void* p, int align, const char* name) {
  if (!p) return fail(XLBG_ERR_ARG, "%s is NULL", name);
  if (((uintptr_t)p) % (uintptr_t)align) return fail(XLBG_ERR_ALIGN, "%s is not %d-byte aligned", name, align);
  return XLBG_OK;
}

static void internal_dims(const xlbg_desc* d, int& n0, int& n1, int& n2) {
  if (d->lattice == XLBG_D2Q9) {
    n0 = 1;
    n1 = (int)d->nx;
    n2 = (int)d->ny;
  } else {
    n0 = (int)d->nx;
    n1 = (int)d->ny;
    n2 = (int)d->nz;
  }
}

static long long ncells(const xlbg_desc* d) { return d->nx * d->ny * d->nz; }

// ---------------------------------------------------------------------------
// set-up kernels
// ---------------------------------------------------------------------------

template <int Q>
__global__ void pack_missing_kernel(const uint8_t* __restrict__ m, uint32_t* __restrict__ bits, long long n) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    uint32_t b = 0;
#pragma unroll
    for (int l = 0; l < Q; ++l) b |= (m[(long long)l * n + c] != 0 ? 1u : 0u) << l;
    bits[c] = b;
  }
}

template <class L, int SK, class T>
__global__ void equilibrium_kernel(const T* __restrict__ rho, const T* __restrict__ u, double rho0, double u00,
                                   double u01, double u02, typename Store<SK, T>::Bits* __restrict__ f, long long n) {
  using St = Store<SK, T>;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const double u0[3] = {u00, u01, u02};
    T r = rho ? rho[c] : T(rho0);
    T uu[L::D];
#pragma unroll
    for (int d = 0; d < L::D; ++d) uu[d] = u ? u[(long long)d * n + c] : T(u0[d]);
    const T usqr = usqr_of<L>(uu);
#pragma unroll
    for (int l = 0; l < L::Q; ++l)
      f[(long long)l * n + c] = St::enc(feq_l<L>(l, r, uu, usqr), T(weight<L>(l)));
  }
}

template <class L, int SK, class T>
__global__ void macroscopic_kernel(const typename Store<SK, T>::Bits* __restrict__ f, T* __restrict__ rho,
                                   T* __restrict__ u, long long n) {
  using St = Store<SK, T>;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    T fl[L::Q];
#pragma unroll
    for (int l = 0; l < L::Q; ++l) fl[l] = St::dec(f[(long long)l * n + c], T(weight<L>(l)));
    T r, uu[L::D];
    macroscopic<L>(fl, r, uu);
    rho[c] = r;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[(long long)d * n + c] = uu[d];
  }
}

// Aux recovery (nse_stepper.py:318-342): slot 0 and the slots opposite to every
// missing direction are copied from f1 (read before the step overwrites it)
// into f0 (written after every pull of the step).  Bit copies of the stored
// values.
template <class L, class Bits>
__global__ void recovery_save_kernel(const Bits* __restrict__ f1, const long long* __restrict__ cells,
                                     const uint32_t* __restrict__ miss, Bits* __restrict__ scratch, long long nrec,
                                     long long n) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nrec;
       r += (long long)gridDim.x * blockDim.x) {
    const long long c = cells[r];
    const uint32_t m = miss[c];
    scratch[r * L::Q] = f1[c];
#pragma unroll
    for (int l = 1; l < L::Q; ++l)
      if ((m >> l) & 1u) scratch[r * L::Q + opp<L>(l)] = f1[(long long)opp<L>(l) * n + c];
  }
}

template <class L, class Bits>
__global__ void recovery_restore_kernel(Bits* __restrict__ f0, const long long* __restrict__ cells,
                                        const uint32_t* __restrict__ miss, const Bits* __restrict__ scratch,
                                        long long nrec, long long n) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nrec;
       r += (long long)gridDim.x * blockDim.x) {
    const long long c = cells[r];
    const uint32_t m = miss[c];
    f0[c] = scratch[r * L::Q];
#pragma unroll
    for (int l = 1; l < L::Q; ++l)
      if ((m >> l) & 1u) f0[(long long)opp<L>(l) * n + c] = scratch[r * L::Q + opp<L>(l)];
  }
}

// Sums the kDiagSlots x 4 block partials into diag[0..3] and clears the slots.
__global__ void diag_finalize_kernel(double* __restrict__ slots, double* __restrict__ diag) {
  __shared__ double red[32][4];
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = threadIdx.x; s < kDiagSlots; s += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] += slots[s * 4 + k];
      slots[s * 4 + k] = 0.0;
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double x = lane < nw ? red[lane][k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) diag[k] = x;
    }
  }
}

// The finaliser launched on its own (the standalone force operator).
int launch_diag_finalize(double* slots, double* out, cudaStream_t s) {
  diag_finalize_kernel<<<1, 1024, 0, s>>>(slots, out);
  return (int)cudaGetLastError();
}

static unsigned grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  if (g > 152LL * 64) g = 152LL * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

template <class L, class Bits>
static void launch_recovery(bool save, void* f, const int64_t* cells, const uint32_t* miss, void* scratch,
                            long long nrec, long long n, cudaStream_t s) {
  const unsigned g = grid_for(nrec, 128);
  if (save)
    recovery_save_kernel<L, Bits><<<g, 128, 0, s>>>((const Bits*)f, (const long long*)cells, miss, (Bits*)scratch,
                                                    nrec, n);
  else
    recovery_restore_kernel<L, Bits><<<g, 128, 0, s>>>((Bits*)f, (const long long*)cells, miss,
                                                       (const Bits*)scratch, nrec, n);
}

template <class L>
static void recovery_by_size(int bytes, bool save, void* f, const int64_t* cells, const uint32_t* miss,
                             void* scratch, long long nrec, long long n, cudaStream_t s) {
  if (bytes == 8)
    launch_recovery<L, unsigned long long>(save, f, cells, miss, scratch, nrec, n, s);
  else if (bytes == 4)
    launch_recovery<L, uint32_t>(save, f, cells, miss, scratch, nrec, n, s);
  else
    launch_recovery<L, unsigned short>(save, f, cells, miss, scratch, nrec, n, s);
}

static void recovery_pass(const xlbg_desc* d, bool save, void* f, const int64_t* cells, const uint32_t* miss,
                          void* scratch, long long nrec, cudaStream_t s) {
  const int bytes = store_bytes(d->store);
  const long long n = ncells(d);
  if (d->lattice == 0)
    recovery_by_size<Lattice<0>>(bytes, save, f, cells, miss, scratch, nrec, n, s);
  else if (d->lattice == 1)
    recovery_by_size<Lattice<1>>(bytes, save, f, cells, miss, scratch, nrec, n, s);
  else
    recovery_by_size<Lattice<2>>(bytes, save, f, cells, miss, scratch, nrec, n, s);
}

// Kernel forced by xlbg_debug_force_kernel (XLBG_KERNEL_*); 0 = automatic.
static std::atomic<int> g_force_kernel{XLBG_KERNEL_AUTO};

int fill_step_args(const xlbg_desc* d, const void* f0, void* f1, const uint8_t* bc_mask,
                          const uint32_t* miss, double omega, StepArgs& a) {
  a.f0 = f0;
  a.f1 = f1;
  a.aux = f1;
  a.bc_mask = bc_mask;
  a.miss = miss;
  a.ncell = ncells(d);
  const int force = g_force_kernel.load();
  a.wide = force == XLBG_KERNEL_MARCH_WIDE || force == XLBG_KERNEL_TMA_WIDE ||
           (long long)lattice_q(d->lattice) * a.ncell > 0xffffffffLL;
  internal_dims(d, a.n0, a.n1, a.n2);
  a.nbc = d->nbc;
  a.omega = omega;
  a.omega_f = (float)omega;
  // cs = compute_dtype(1.0 / wp.sqrt(3.0)) with wp.sqrt evaluated in float32 at
  // Python scope (bc_extrapolation_outflow.py:353)
  a.extrap_cs = 1.0 / (double)sqrtf(3.0f);
  for (int b = 0; b < kMaxBC; ++b) {
    if (b < d->nbc) {
      a.bc[b].id = d->bc[b].id;
      a.bc[b].kind = d->bc[b].kind;
      a.bc[b].rho = d->bc[b].rho;
      a.bc[b].u[0] = d->bc[b].u[0];
      a.bc[b].u[1] = d->bc[b].u[1];
      a.bc[b].u[2] = d->bc[b].u[2];
    } else {
      a.bc[b].id = -1;
      a.bc[b].kind = 0;
      a.bc[b].rho = 0.0;
      a.bc[b].u[0] = a.bc[b].u[1] = a.bc[b].u[2] = 0.0;
    }
  }
  for (int i = 0; i < 256; ++i) a.bc_code[i] = 0;
  for (int b = 0; b < d->nbc; ++b) a.bc_code[d->bc[b].id & 0xff] = (uint16_t)(d->bc[b].kind | (b << 8));
  a.force_id = -1;
  a.diag_slots = nullptr;
  a.timestep = 0;
  return XLBG_OK;
}

// Rows per thread of the marching kernel: at least eight blocks per SM of a
// 152-SM GB300 and at most 32 rows per thread (D3Q19 FP32 at 512^3: 64 rows
// 41.2-41.7, 32 rows 41.7, 16 rows 41.8 GLUPS: within run-to-run spread).
static int choose_chunk(const StepArgs& a, int threads) {
  const long long columns = (long long)a.n0 * ((a.n2 + threads - 1) / threads);
  long long chunk = (long long)a.n1 * columns / (152LL * 8);
  if (chunk < 1) chunk = 1;
  if (chunk > 32) chunk = 32;
  return (int)chunk;
}

int try_launch_tma(const xlbg_desc* d, const StepArgs& a, bool fullbc, bool diag, cudaStream_t s);

int launch_main(const xlbg_desc* d, const StepArgs& a, bool diag, cudaStream_t s) {
  const bool full = needs_full_bc(d) || diag;
  const int force = g_force_kernel.load();
  // 16-bit stores: TMA-staged rows when the shape allows (1 = not applicable)
  if (force == XLBG_KERNEL_AUTO || force == XLBG_KERNEL_TMA_WIDE) {
    const int t = try_launch_tma(d, a, full, diag, s);
    if (t != 1) return t;
  }
  const int pair = d->collision == XLBG_KBC ? 0 : d->collision;  // BGK form: 0, 2 or 3
  int r = -1;
  // the marching kernel keeps cell offsets in 32 bits (plane offsets are 64-bit when a.wide)
  if (a.ncell < 0x7fffffffLL && force != XLBG_KERNEL_CELL) {
    const int threads = a.n2 >= kStepBlock ? kStepBlock : ((a.n2 + 31) / 32) * 32;
    const int chunk = choose_chunk(a, threads);
    if (chunk > 0) {
      if (d->lattice == 0)
        r = d->collision == XLBG_KBC ? launch_step_march_d2q9_kbc(a, d->store, d->compute, full, threads, chunk, s)
                                     : launch_step_march_d2q9_bgk(a, d->store, d->compute, full, pair, threads, chunk, s);
      else if (d->lattice == 1)
        r = launch_step_march_d3q19_bgk(a, d->store, d->compute, full, pair, threads, chunk, s);
      else
        r = d->collision == XLBG_KBC ? launch_step_march_d3q27_kbc(a, d->store, d->compute, full, threads, chunk, s)
                                     : launch_step_march_d3q27_bgk(a, d->store, d->compute, full, pair, threads, chunk, s);
      if (r < 0) return fail(XLBG_ERR_UNSUPPORTED, "store/compute pair not supported");
      return cuda_status((cudaError_t)r, "step kernel launch");
    }
  }
  if (d->lattice == 0)
    r = d->collision == XLBG_KBC ? launch_step_d2q9_kbc(a, d->store, d->compute, full, diag, s)
                                 : launch_step_d2q9_bgk(a, d->store, d->compute, full, diag, pair, s);
  else if (d->lattice == 1)
    r = launch_step_d3q19_bgk(a, d->store, d->compute, full, diag, pair, s);
  else
    r = d->collision == XLBG_KBC ? launch_step_d3q27_kbc(a, d->store, d->compute, full, diag, s)
                                 : launch_step_d3q27_bgk(a, d->store, d->compute, full, diag, pair, s);
  if (r < 0) return fail(XLBG_ERR_UNSUPPORTED, "store/compute pair not supported");
  return cuda_status((cudaError_t)r, "step kernel launch");
}

int check_step_args(const xlbg_desc* d, const void* f0, const void* f1, const uint8_t* bc_mask,
                           const uint32_t* miss, const int64_t* rec_cells, int64_t n_rec, const void* rec_scratch) {
  int e;
  if ((e = check_desc(d))) return e;
  const int sb = store_bytes(d->store);
  if ((e = check_ptr(f0, sb, "f0"))) return e;
  if ((e = check_ptr(f1, sb, "f1"))) return e;
  if (f0 == f1) return fail(XLBG_ERR_ARG, "f0 and f1 must be distinct buffers");
  if ((e = check_ptr(bc_mask, 1, "bc_mask"))) return e;
  if ((e = check_ptr(miss, 4, "miss_bits"))) return e;
  if (n_rec < 0) return fail(XLBG_ERR_ARG, "n_rec < 0");
  if (n_rec > 0) {
    if ((e = check_ptr(rec_cells, 8, "rec_cells"))) return e;
    if ((e = check_ptr(rec_scratch, sb, "rec_scratch"))) return e;
  }
  return XLBG_OK;
}

int one_step(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
                    const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, bool diag,
                    int force_id, double* slots, double* out, cudaStream_t s, int timestep) {
  StepArgs a;
  fill_step_args(d, f0, f1, bc_mask, miss, omega, a);
  a.timestep = (unsigned)timestep;
  a.force_id = force_id;
  a.diag_slots = slots;
  if (n_rec > 0) recovery_pass(d, true, f1, rec_cells, miss, rec_scratch, n_rec, s);
  int e = launch_main(d, a, diag, s);
  if (e) return e;
  if (n_rec > 0) recovery_pass(d, false, f0, rec_cells, miss, rec_scratch, n_rec, s);
  if (diag) diag_finalize_kernel<<<1, 1024, 0, s>>>(slots, out);
  return cuda_status(cudaGetLastError(), "step launch");
}

}  // namespace xlbg

namespace xlbg {

template <class L>
static int tables_for(int32_t* c, double* w, int32_t* o) {
  for (int l = 0; l < L::Q; ++l) {
    for (int k = 0; k < L::D; ++k) c[l * L::D + k] = L::c(l, k);
    w[l] = weight<L>(l);
    o[l] = opp<L>(l);
  }
  return L::Q;
}

template <class L, int SK, class T>
static int eq_launch(const xlbg_desc* d, const void* rho, const void* u, double rho0, const double* u0, void* f,
                     cudaStream_t s) {
  const long long n = ncells(d);
  const double a = u0 ? u0[0] : 0.0, b = u0 ? u0[1] : 0.0, c = (u0 && L::D == 3) ? u0[2] : 0.0;
  equilibrium_kernel<L, SK, T><<<grid_for(n, 256), 256, 0, s>>>(
      (const T*)rho, (const T*)u, rho0, a, b, c, (typename Store<SK, T>::Bits*)f, n);
  return cuda_status(cudaGetLastError(), "equilibrium launch");
}

template <class L, int SK, class T>
static int macro_launch(const xlbg_desc* d, const void* f, void* rho, void* u, cudaStream_t s) {
  const long long n = ncells(d);
  macroscopic_kernel<L, SK, T><<<grid_for(n, 256), 256, 0, s>>>((const typename Store<SK, T>::Bits*)f, (T*)rho,
                                                                (T*)u, n);
  return cuda_status(cudaGetLastError(), "macroscopic launch");
}

#define XLBG_LSC_DISPATCH(CALL, ...)                                                      \
  do {                                                                                    \
    const int sk = d->store;                                                              \
    if (d->compute == XLBG_COMPUTE_F64) {                                                 \
      if (sk == SK_F64) return CALL<L, SK_F64, double>(__VA_ARGS__);                     \
      if (sk == SK_F32) return CALL<L, SK_F32, double>(__VA_ARGS__);                     \
      if (sk == SK_F16) return CALL<L, SK_F16, double>(__VA_ARGS__);                     \
    } else {                                                                              \
      if (sk == SK_F32) return CALL<L, SK_F32, float>(__VA_ARGS__);                      \
      if (sk == SK_F16) return CALL<L, SK_F16, float>(__VA_ARGS__);                      \
      if (sk == SK_F16S) return CALL<L, SK_F16S, float>(__VA_ARGS__);                    \
      if (sk == SK_BF16S) return CALL<L, SK_BF16S, float>(__VA_ARGS__);                  \
    }                                                                                     \
    return fail(XLBG_ERR_UNSUPPORTED, "store/compute pair not supported");                \
  } while (0)

template <class L>
static int eq_by_lattice(const xlbg_desc* d, const void* rho, const void* u, double rho0, const double* u0, void* f,
                         cudaStream_t s) {
  XLBG_LSC_DISPATCH(eq_launch, d, rho, u, rho0, u0, f, s);
}

template <class L>
static int macro_by_lattice(const xlbg_desc* d, const void* f, void* rho, void* u, cudaStream_t s) {
  XLBG_LSC_DISPATCH(macro_launch, d, f, rho, u, s);
}

}  // namespace xlbg

using namespace xlbg;

extern "C" {

int xlbg_abi_version(void) { return XLBG_ABI_VERSION; }

int xlbg_debug_force_kernel(int32_t kernel) {
  if (kernel < XLBG_KERNEL_AUTO || kernel > XLBG_KERNEL_TMA_WIDE)
    return fail(XLBG_ERR_ARG, "unknown kernel selector %d", kernel);
  g_force_kernel.store(kernel);
  return XLBG_OK;
}

const char* xlbg_last_error(void) { return g_last_error.c_str(); }

int xlbg_lattice_tables(int32_t lattice, int32_t* c, double* w, int32_t* opp_out) {
  if (!c || !w || !opp_out) return -fail(XLBG_ERR_ARG, "NULL output");
  if (lattice == 0) return tables_for<Lattice<0>>(c, w, opp_out);
  if (lattice == 1) return tables_for<Lattice<1>>(c, w, opp_out);
  if (lattice == 2) return tables_for<Lattice<2>>(c, w, opp_out);
  return -fail(XLBG_ERR_ARG, "unknown lattice %d", lattice);
}

int xlbg_pack_missing(const xlbg_desc* d, const uint8_t* missing_mask, uint32_t* miss_bits, void* stream) {
  int e;
  if ((e = check_desc(d))) return e;
  if ((e = check_ptr(missing_mask, 1, "missing_mask"))) return e;
  if ((e = check_ptr(miss_bits, 4, "miss_bits"))) return e;
  const long long n = ncells(d);
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned g = grid_for(n, 256);
  if (d->lattice == 0)
    pack_missing_kernel<9><<<g, 256, 0, s>>>(missing_mask, miss_bits, n);
  else if (d->lattice == 1)
    pack_missing_kernel<19><<<g, 256, 0, s>>>(missing_mask, miss_bits, n);
  else
    pack_missing_kernel<27><<<g, 256, 0, s>>>(missing_mask, miss_bits, n);
  return cuda_status(cudaGetLastError(), "pack_missing launch");
}

int xlbg_step(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
              const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep,
              void* stream) {
  int e;
  if ((e = check_step_args(d, f0, f1, bc_mask, miss, rec_cells, n_rec, rec_scratch))) return e;
  return one_step(d, f0, f1, bc_mask, miss, rec_cells, n_rec, rec_scratch, omega, false, -1, nullptr, nullptr,
                  (cudaStream_t)stream, timestep);
}

int xlbg_run(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
             const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep0,
             int32_t n_steps, void* stream) {
  int e;
  if ((e = check_step_args(d, f0, f1, bc_mask, miss, rec_cells, n_rec, rec_scratch))) return e;
  if (n_steps < 0) return fail(XLBG_ERR_ARG, "n_steps < 0");
  void* a = f0;
  void* b = f1;
  for (int k = 0; k < n_steps; ++k) {
    if ((e = one_step(d, a, b, bc_mask, miss, rec_cells, n_rec, rec_scratch, omega, false, -1, nullptr, nullptr,
                      (cudaStream_t)stream, timestep0 + k)))
      return e;
    void* t = a;
    a = b;
    b = t;
  }
  return XLBG_OK;
}

int xlbg_step_diag(const xlbg_desc* d, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss,
                   const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep,
                   int32_t force_id, double* diag_slots, double* diag, void* stream) {
  int e;
  if ((e = check_step_args(d, f0, f1, bc_mask, miss, rec_cells, n_rec, rec_scratch))) return e;
  if ((e = check_ptr(diag_slots, 8, "diag_slots"))) return e;
  if ((e = check_ptr(diag, 8, "diag"))) return e;
  return one_step(d, f0, f1, bc_mask, miss, rec_cells, n_rec, rec_scratch, omega, true, force_id, diag_slots, diag,
                  (cudaStream_t)stream, timestep);
}

int xlbg_equilibrium(const xlbg_desc* d, const void* rho, const void* u, double rho0, const double* u0, void* f,
                     void* stream) {
  int e;
  if ((e = check_desc(d))) return e;
  if ((e = check_ptr(f, store_bytes(d->store), "f"))) return e;
  cudaStream_t s = (cudaStream_t)stream;
  if (d->lattice == 0) return eq_by_lattice<Lattice<0>>(d, rho, u, rho0, u0, f, s);
  if (d->lattice == 1) return eq_by_lattice<Lattice<1>>(d, rho, u, rho0, u0, f, s);
  return eq_by_lattice<Lattice<2>>(d, rho, u, rho0, u0, f, s);
}

int xlbg_macroscopic(const xlbg_desc* d, const void* f, void* rho, void* u, void* stream) {
  int e;
  if ((e = check_desc(d))) return e;
  if ((e = check_ptr(f, store_bytes(d->store), "f"))) return e;
  const int tb = d->compute == XLBG_COMPUTE_F64 ? 8 : 4;
  if ((e = check_ptr(rho, tb, "rho"))) return e;
  if ((e = check_ptr(u, tb, "u"))) return e;
  cudaStream_t s = (cudaStream_t)stream;
  if (d->lattice == 0) return macro_by_lattice<Lattice<0>>(d, f, rho, u, s);
  if (d->lattice == 1) return macro_by_lattice<Lattice<1>>(d, f, rho, u, s);
  return macro_by_lattice<Lattice<2>>(d, f, rho, u, s);
}

}  // extern "C"
