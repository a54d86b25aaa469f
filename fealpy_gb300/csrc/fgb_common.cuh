// Shared device helpers for the FEALPy GB300 kernels (sm_103a).
//
// Conventions used by every kernel in this library:
//   * every pointer argument is a device pointer unless its name ends in _host;
//   * kernels never trap: an inconsistency found on the device (an index out of
//     range, a column missing from a row pattern, a non-finite scalar) is
//     recorded in a caller-provided int32 status word with atomicMax and the
//     offending access is skipped;
//   * all reductions are deterministic: partial sums are written per block and
//     combined in a fixed order by the last block to finish (no floating-point
//     atomics anywhere).
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/fealpy_gb300.h"

namespace fgb {

constexpr int kWarp = 32;
constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs (only used as a grid-size hint)
// Longest row whose within-row column positions the hashed pattern pass
// records (one byte per contribution); the numeric pass indexes rows up to
// this length directly and searches the columns of longer ones.
constexpr int kRowMapMax = 128;

__device__ __forceinline__ void set_status(int32_t* status, int32_t code) {
  if (status) atomicMax(status, code);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T group_sum(T v, int width) {
  for (int o = width >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, width);
  return v;
}

// Block-wide sum with a fixed combination order (warp shuffles, then warp 0
// over the per-warp results).  Result valid in thread 0.  `smem` needs
// blockDim.x/32 entries.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* smem) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) smem[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  T r = (threadIdx.x < nw) ? smem[threadIdx.x] : T(0);
  if (wid == 0) r = warp_sum(r);
  return r;
}

// Streaming loads for matrix data that is touched once per sweep: mark the
// lines evict-first so that the Krylov vectors stay resident in the 129 MB L2.
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int32_t ld_stream(const int32_t* p) { return __ldcs(p); }
__device__ __forceinline__ int64_t ld_stream(const int64_t* p) {
  return static_cast<int64_t>(__ldcs(reinterpret_cast<const long long*>(p)));
}

// lower_bound over a sorted int32 array held in shared memory.
__device__ __forceinline__ int lower_bound_i32(const int32_t* a, int n, int32_t key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int lower_bound_i32_global(const int32_t* a, int64_t n, int32_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
  }
  return static_cast<int>(lo);
}

inline int grid_for(int64_t work, int per_block, int cap = 1 << 20) {
  int64_t g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return static_cast<int>(g);
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FGB_OK : FGB_ERR_CUDA;
}

__host__ __device__ inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Carves sub-buffers out of a caller-provided workspace.
struct Carver {
  char* base;
  size_t size;
  size_t off = 0;
  bool ok = true;
  Carver(void* b, size_t s) : base(static_cast<char*>(b)), size(s) {}
  template <typename T>
  T* take(size_t count) {
    size_t bytes = align_up(count * sizeof(T));
    if (off + bytes > size || base == nullptr) { ok = false; return nullptr; }
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
};

// ---------------------------------------------------------------------------
// Exclusive scan of int32 counts into int64 offsets (out has n+1 entries).
// Three launches: per-tile sums, a single-block scan of the tile sums, and the
// per-tile scan with the tile offset added.  Workspace: fgb_scan_workspace_bytes.
// ---------------------------------------------------------------------------
int exclusive_scan_i32_to_i64(const int32_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes,
                              cudaStream_t stream);
size_t scan_workspace_bytes(int64_t n);

}  // namespace fgb
