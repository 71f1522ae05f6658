// scan.cuh — block-wide and device-wide exclusive scans shared by the
// schedule builder and the contour tracer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace bf {

constexpr uint32_t SCAN_TPB = 1024;
constexpr uint32_t SCAN_ITEMS = 4;  // elements per thread of a scan block
constexpr uint32_t SCAN_BLOCK = SCAN_TPB * SCAN_ITEMS;

// Block-wide exclusive scan of one value per thread (SCAN_TPB threads).
template <class T>
__device__ __forceinline__ T block_exscan(T v, T* total) {
  __shared__ T wsum[SCAN_TPB / 32];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T s = lane < SCAN_TPB / 32 ? wsum[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    if (lane < SCAN_TPB / 32) wsum[lane] = s;
  }
  __syncthreads();
  const T before = (wid ? wsum[wid - 1] : T(0)) + x - v;
  *total = wsum[SCAN_TPB / 32 - 1];
  __syncthreads();
  return before;
}

// Values of the two scans: live-bit popcounts of bitmap words, and per-row
// (edges | items << 32).
struct PopVal {
  const uint32_t* a;
  __device__ uint32_t operator()(uint64_t i) const { return __popc(a[i]); }
};
struct U64Val {
  const uint64_t* a;
  __device__ uint64_t operator()(uint64_t i) const { return a[i]; }
};

// Three-phase exclusive scan over m elements (m read from *mp when mp is
// set, else the argument): block sums, a scan of the block sums in one
// block, then each block's own scan. out[m] receives the total.
template <class T, class V>
__global__ void __launch_bounds__(SCAN_TPB) k_scan_sums(V val, uint64_t m0, const uint32_t* mp,
                                                        T* __restrict__ bsum) {
  const uint64_t m = mp ? *mp : m0;
  const uint64_t b0 = (uint64_t)blockIdx.x * SCAN_BLOCK;
  T s = 0;
  for (uint32_t j = 0; j < SCAN_ITEMS; ++j) {
    const uint64_t i = b0 + (uint64_t)j * SCAN_TPB + threadIdx.x;
    if (i < m) s += val(i);
  }
  T tot;
  block_exscan<T>(s, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

template <class T>
__global__ void __launch_bounds__(SCAN_TPB) k_scan_top(T* __restrict__ bsum, uint32_t nb) {
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t b0 = 0; b0 < nb; b0 += SCAN_TPB) {
    const uint32_t i = b0 + threadIdx.x;
    const T v = i < nb ? bsum[i] : T(0);
    T tot;
    const T ex = block_exscan<T>(v, &tot);
    const T c = carry;
    if (i < nb) bsum[i] = c + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

template <class T, class V>
__global__ void __launch_bounds__(SCAN_TPB) k_scan_out(V val, uint64_t m0, const uint32_t* mp,
                                                       const T* __restrict__ bsum, uint32_t nb,
                                                       T* __restrict__ out) {
  const uint64_t m = mp ? *mp : m0;
  const uint64_t b0 = (uint64_t)blockIdx.x * SCAN_BLOCK;
  // thread t scans elements b0 + t * SCAN_ITEMS .. + SCAN_ITEMS - 1 (contiguous)
  T v[SCAN_ITEMS];
  T s = 0;
  for (uint32_t j = 0; j < SCAN_ITEMS; ++j) {
    const uint64_t i = b0 + (uint64_t)threadIdx.x * SCAN_ITEMS + j;
    v[j] = i < m ? val(i) : T(0);
    s += v[j];
  }
  T tot;
  T run = bsum[blockIdx.x] + block_exscan<T>(s, &tot);
  for (uint32_t j = 0; j < SCAN_ITEMS; ++j) {
    const uint64_t i = b0 + (uint64_t)threadIdx.x * SCAN_ITEMS + j;
    if (i < m) out[i] = run;
    run += v[j];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[m] = bsum[nb];
}


// Exclusive scan of m elements val(0 .. m) into out[0 .. m] (out[m] = total)
// with nb = ceil(m / SCAN_BLOCK) blocks and bsum room for nb + 1 sums.
template <class T, class V>
inline void scan_launch(V val, uint64_t m, T* bsum, T* out, cudaStream_t st) {
  const unsigned nb = (unsigned)std::max<uint64_t>(1, (m + SCAN_BLOCK - 1) / SCAN_BLOCK);
  k_scan_sums<T><<<nb, SCAN_TPB, 0, st>>>(val, m, nullptr, bsum);
  k_scan_top<T><<<1, SCAN_TPB, 0, st>>>(bsum, nb);
  k_scan_out<T><<<nb, SCAN_TPB, 0, st>>>(val, m, nullptr, bsum, nb, out);
}

}  // namespace bf
