// crg_peaks.cu -- arithmetic diagnostics of the current device.
//
// FP64 / FP32 fused-multiply-add throughput: the force kernels are bound by the FP64 (plain
// path) or FP32 (mixed path) pipes rather than by HBM, so their roofline needs these two
// peaks.  Each thread runs 8 independent dependent chains x = x * a + b; the grid covers
// every SM many times over.
//
// Division check: div_rn_recip (the division from a correctly rounded reciprocal that the
// rod pass kernel uses) against the IEEE division, bit for bit, on generated operands.
#include <cuda_runtime.h>

#include <algorithm>

#include "crg_internal.cuh"
#include "crg_kernels.h"
#include "../../include/crg.h"

namespace crg {

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)-1.25) out[0] = s;  // never true; keeps the chains alive
}

template <typename T>
int run_one(double *tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CRG_ECUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CRG_ECUDA;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return CRG_ENOMEM;
  const int threads = 256;
  const int blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 1024;
  float ms = 0.f;
  const T a = (T)0.999999, b = (T)1e-7;
  // grow the iteration count until one launch takes at least 40 ms
  for (int attempt = 0; attempt < 24; ++attempt) {
    k_fma_chains<T><<<blocks, threads>>>(out, iters, a, b);  // warm-up
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, threads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms >= 40.f || iters >= (1 << 26)) break;
    iters *= (ms < 1.f) ? 8 : 2;
  }
  const double flops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? CRG_OK : CRG_ECUDA;
}

}  // namespace

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double u01(uint64_t r) { return (double)(r >> 11) * 0x1.0p-53; }

// A double of the given sign, biased exponent and 52-bit fraction.
__device__ __forceinline__ double make_f64(uint64_t sign, uint64_t bexp, uint64_t frac) {
  return __longlong_as_double((long long)((sign << 63) | (bexp << 52) | (frac & ((1ull << 52) - 1))));
}

// Operands of case k % 5: 0 rod-like (|a| < 100, b in [0.01, 100)); 1 random signs,
// fractions and biased exponents 600..1446 (across the fast path's bounds); 2 quotients
// near the midpoint between two doubles (a = b (q + ulp(q) / 2), then moved by -2..2 ulp);
// 3 divisors with an all-ones fraction or a power of two; 4 squared norms and dot products
// as the rod kernels form them (segment vectors of length 1-6 in random directions).
__global__ void k_check_division(int64_t n, uint64_t seed, unsigned long long *bad,
                                 unsigned long long *fast) {
  unsigned long long nb = 0, nf = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r0 = mix64(seed ^ mix64((uint64_t)k)), r1 = mix64(r0), r2 = mix64(r1);
    double a, b;
    switch ((int)(k % 5)) {
      case 0:
        a = (u01(r0) - 0.5) * 200.0;
        b = 0.01 + u01(r1) * 100.0;
        break;
      case 1:
        a = make_f64(r0 >> 63, 600 + (r1 >> 32) % 847, r2);
        b = make_f64((r1 >> 31) & 1, 600 + (r2 >> 40) % 847, r0);
        break;
      case 2: {
        const double q = make_f64(r0 >> 63, 1023 - 40 + (r1 >> 40) % 81, r2);
        b = make_f64(0, 1023 - 40 + (r2 >> 48) % 81, r1);
        const double h = __dmul_rn(__longlong_as_double(__double_as_longlong(q) & 0xfff0000000000000ll), 0x1.0p-53);
        a = __fma_rn(b, h, __dmul_rn(b, q));
        a = __longlong_as_double(__double_as_longlong(a) + (long long)((r0 >> 8) % 5) - 2);
        break;
      }
      case 3:
        a = (u01(r0) - 0.5) * 64.0;
        b = make_f64(0, 1023 - 60 + (r1 >> 40) % 121, (r2 & 1) ? ~0ull : 0ull);
        break;
      default: {
        const double len = 1.0 + 5.0 * u01(r0), ang = 6.283185307179586 * u01(r1);
        const double ab0 = len * cos(ang), ab1 = len * sin(ang);
        const double ap0 = (u01(r2) - 0.5) * 20.0, ap1 = (u01(mix64(r2)) - 0.5) * 20.0;
        a = __dadd_rn(__dmul_rn(ab0, ap0), __dmul_rn(ab1, ap1));
        b = __dadd_rn(__dmul_rn(ab0, ab0), __dmul_rn(ab1, ab1));
        break;
      }
    }
    const double y = __drcp_rn(b);
    const double got = div_rn_recip(a, b, y), want = __ddiv_rn(a, b);
    nb += __double_as_longlong(got) != __double_as_longlong(want);
    const unsigned long long ea = ((unsigned long long)__double_as_longlong(a) >> 52) & 0x7ffull;
    const unsigned long long eb = ((unsigned long long)__double_as_longlong(b) >> 52) & 0x7ffull;
    nf += (ea - 623ull <= 800ull && eb - 623ull <= 800ull);
  }
  atomicAdd(bad, nb);
  atomicAdd(fast, nf);
}

}  // namespace

int check_division(int64_t n, uint64_t seed, int64_t *mismatches, int64_t *fast) {
  unsigned long long *d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return CRG_ENOMEM;
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemset(d, 0, sizeof(h));
  if (e == cudaSuccess) {
    k_check_division<<<152 * 8, 256>>>(n, seed, d, d + 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  *mismatches = (int64_t)h[0];
  *fast = (int64_t)h[1];
  return e == cudaSuccess ? CRG_OK : CRG_ECUDA;
}

int measure_fma_peaks(double *fp64_tflops, double *fp32_tflops) {
  int r = run_one<double>(fp64_tflops);
  if (r != CRG_OK) return r;
  return run_one<float>(fp32_tflops);
}

}  // namespace crg
