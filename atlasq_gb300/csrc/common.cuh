// Shared device helpers for the GB300 MPS kernels (sm_103a).
// Complex values are interleaved (re, im): float2 for complex64, double2 for
// complex128 -- the layout of torch.complex64 / torch.complex128 storage.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "atlasq_gb300.h"

#define AGB_HD __host__ __device__ __forceinline__
#define AGB_DEV __device__ __forceinline__

template <typename CX> struct cx_traits;
template <> struct cx_traits<float2> { typedef float R; };
template <> struct cx_traits<double2> { typedef double R; };

template <typename CX> AGB_HD CX mk(typename cx_traits<CX>::R re, typename cx_traits<CX>::R im) {
  CX z;
  z.x = re;
  z.y = im;
  return z;
}
template <typename CX> AGB_HD CX czero() { return mk<CX>(0, 0); }
template <typename CX> AGB_HD CX cmul(CX a, CX b) { return mk<CX>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// conj(a) * b
template <typename CX> AGB_HD CX cmulc(CX a, CX b) { return mk<CX>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
template <typename CX> AGB_HD CX cadd(CX a, CX b) { return mk<CX>(a.x + b.x, a.y + b.y); }
template <typename CX> AGB_HD CX csub(CX a, CX b) { return mk<CX>(a.x - b.x, a.y - b.y); }
template <typename CX> AGB_HD CX cconj(CX a) { return mk<CX>(a.x, -a.y); }
template <typename CX> AGB_HD CX cscale(CX a, typename cx_traits<CX>::R s) { return mk<CX>(a.x * s, a.y * s); }
template <typename CX> AGB_HD typename cx_traits<CX>::R cabs2(CX a) { return a.x * a.x + a.y * a.y; }
// 1 / z
template <typename CX> AGB_HD CX cinv(CX z) {
  typename cx_traits<CX>::R d = z.x * z.x + z.y * z.y;
  return mk<CX>(z.x / d, -z.y / d);
}
// acc += a * b
template <typename CX> AGB_HD void cfma(CX& acc, CX a, CX b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename CX> AGB_HD void cfmac(CX& acc, CX a, CX b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}

template <typename T> AGB_DEV T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename CX> AGB_DEV CX warp_csum(CX v) {
  v.x = warp_sum(v.x);
  v.y = warp_sum(v.y);
  return v;
}

// Sum of float terms with double-precision accuracy.  The running sum is an
// unevaluated pair hi + lo updated by Knuth's TwoSum (error-free: hi + x =
// s + e exactly) and products enter through the FMA error-free product
// (a * b = p + fma(a, b, -p) exactly), so the accumulation runs on the FP32
// pipe.  GB300 issues about 2 FP64 operations per SM per clock, 64x fewer than
// FP32, which makes plain double accumulation the bottleneck of any pass over
// a matrix.  The double specialisation is plain double arithmetic.
template <typename R> struct SumAcc;
template <> struct SumAcc<float> {
  float hi = 0.f, lo = 0.f;
  AGB_DEV void merge(float x, float xlo) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, xlo), e);
  }
  AGB_DEV void add(float x) { merge(x, 0.f); }
  AGB_DEV void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    merge(p, fmaf(a, b, -p));
  }
  // every lane of the warp ends with the warp's total (TwoSum is exact, so
  // both partners of a butterfly step compute the same pair)
  AGB_DEV void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h = __shfl_xor_sync(0xffffffffu, hi, o), l = __shfl_xor_sync(0xffffffffu, lo, o);
      merge(h, l);
    }
  }
  AGB_DEV double value() const { return (double)hi + (double)lo; }
};
template <> struct SumAcc<double> {
  double s = 0.0;
  AGB_DEV void add(double x) { s += x; }
  AGB_DEV void add_prod(double a, double b) { s = fma(a, b, s); }
  AGB_DEV void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  AGB_DEV double value() const { return s; }
};

// Block-wide sum of one value per thread; `red` must hold >= 32 entries.
// All threads of the block must call it; every thread gets the result.
template <typename T> AGB_DEV T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T t = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  T r = red[0];
  __syncthreads();
  return r;
}

// Block-wide sum of two values at once (one reduction round instead of two).
template <typename T> AGB_DEV void block_sum2(T& a, T& b, T* red /* >= 64 entries */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  __syncthreads();
  if (lane == 0) {
    red[wid] = a;
    red[32 + wid] = b;
  }
  __syncthreads();
  if (wid == 0) {
    T x = (lane < nw) ? red[lane] : T(0);
    T y = (lane < nw) ? red[32 + lane] : T(0);
    x = warp_sum(x);
    y = warp_sum(y);
    if (lane == 0) {
      red[0] = x;
      red[32] = y;
    }
  }
  __syncthreads();
  a = red[0];
  b = red[32];
  __syncthreads();
}

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, SC'11 (Random123).  Same definition as the CPU
// oracle: ten rounds, multipliers 0xD2511F53 / 0xCD9E8D57, Weyl increments
// 0x9E3779B9 / 0xBB67AE85.
struct philox_out {
  uint32_t x, y, z, w;
};
AGB_DEV philox_out philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                  uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  philox_out o;
  o.x = c0;
  o.y = c1;
  o.z = c2;
  o.w = c3;
  return o;
}

// Standard normal from Philox words (Box-Muller on 24-bit uniforms).
AGB_DEV float philox_normal(uint64_t seed, uint64_t idx, uint32_t stream) {
  philox_out o = philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32), stream, 0x5EEDu, (uint32_t)seed,
                               (uint32_t)(seed >> 32));
  const float u1 = ((float)(o.x >> 8) + 1.0f) * (1.0f / 16777216.0f);
  const float u2 = (float)(o.y >> 8) * (1.0f / 16777216.0f);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

AGB_HD size_t agb_align(size_t x) { return (x + 255) & ~(size_t)255; }

// Opts `kern` in to `dyn` bytes of dynamic shared memory when its static plus
// dynamic shared memory exceeds the 48 KiB a launch gets by default (a launch
// over that limit without the opt-in is refused with cudaErrorInvalidValue).
template <typename K>
inline cudaError_t agb_smem_optin(K kern, size_t dyn) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  if (a.sharedSizeBytes + dyn <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

// Counts kernel launches issued by this library (read with agb_launch_count).
void agb_note_launch();
// Records where a launch check failed (read with agb_last_error).
void agb_note_error(const char* file, int line, cudaError_t e);

#define AGB_CHECK_LAUNCH()                      \
  do {                                          \
    agb_note_launch();                          \
    cudaError_t _e = cudaGetLastError();        \
    if (_e != cudaSuccess) {                    \
      agb_note_error(__FILE__, __LINE__, _e);   \
      return AGB_ERR_CUDA;                      \
    }                                           \
  } while (0)
