// The calling thread's current CUDA context, for caches of device addresses.
//
// Device addresses of static __device__ arrays (cudaGetSymbolAddress) belong to
// one context: after cudaDeviceReset the device gets a new primary context and
// the old addresses are gone.  Caches keyed by device ordinal alone would hand
// out stale addresses, so they also keep the context the addresses were looked
// up in and look them up again when it changes.  cuCtxGetCurrent is reached
// through the runtime's driver entry-point query, so the library needs no link
// to libcuda.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace xlbg {

inline void* current_context() {
  typedef CUresult (*GetCurrentFn)(CUcontext*);
  static const GetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<GetCurrentFn>(p);
  }();
  CUcontext c = nullptr;
  if (fn == nullptr || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

}  // namespace xlbg
