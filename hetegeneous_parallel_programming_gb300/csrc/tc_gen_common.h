// Seeded graph generators shared by the host (C++/OpenMP) and the device
// (CUDA) so that both produce bit-identical edge samples.
//
// The random source is counter based: sample i of stream (seed, sid) is a
// pure function of (seed, sid, i), so any thread can draw any sample.  The
// mixing function is the 64-bit finaliser of SplitMix64 (Steele, Lea, Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014).  All
// decisions are made in integer arithmetic from thresholds that the host
// computes once, so no floating-point rounding can differ between CPU and GPU.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define TC_HD __host__ __device__ __forceinline__
#else
#define TC_HD static inline
#endif

TC_HD uint64_t tc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

TC_HD uint64_t tc_stream_key(uint64_t seed, uint64_t sid) {
  return tc_mix64(seed * 0x9E3779B97F4A7C15ULL + sid * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
}

TC_HD uint64_t tc_rand_at(uint64_t key, uint64_t i) { return tc_mix64(key + (i + 1) * 0x9E3779B97F4A7C15ULL); }

// floor(r * n / 2^64): an unbiased-enough map of a 64-bit word onto [0, n).
TC_HD uint64_t tc_mulhi(uint64_t r, uint64_t n) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(r, n);
#else
  return (uint64_t)(((unsigned __int128)r * (unsigned __int128)n) >> 64);
#endif
}

enum { TC_SID_ER = 1, TC_SID_RMAT = 2, TC_SID_RGG = 3, TC_SID_CL = 4 };

// Erdos-Renyi G(n, M): sample i draws two independent uniform endpoints.
TC_HD void tc_er_sample(uint64_t key, uint64_t n, uint64_t i, int32_t *u, int32_t *v) {
  *u = (int32_t)tc_mulhi(tc_rand_at(key, 2 * i), n);
  *v = (int32_t)tc_mulhi(tc_rand_at(key, 2 * i + 1), n);
}

// R-MAT (Chakrabarti, Zhan, Faloutsos, SDM 2004) without noise: at each of
// `scale` levels pick a quadrant with probabilities a, b, c, d from a 32-bit
// uniform compared against integer thresholds t1 < t2 < t3 (= cumulative
// probabilities * 2^32).  The most significant id bit is chosen first.
TC_HD void tc_rmat_sample(uint64_t key, int scale, uint64_t t1, uint64_t t2, uint64_t t3, uint64_t i,
                          int32_t *u, int32_t *v) {
  const uint64_t words = (uint64_t)((scale + 1) / 2);
  uint32_t uu = 0, vv = 0;
  uint64_t w = 0;
  for (int l = 0; l < scale; ++l) {
    if ((l & 1) == 0) w = tc_rand_at(key, i * words + (uint64_t)(l >> 1));
    const uint64_t r = (l & 1) ? (w >> 32) : (w & 0xffffffffULL);
    const uint32_t bu = r >= t2 ? 1u : 0u;
    const uint32_t bv = (r >= t1 && r < t2) || r >= t3 ? 1u : 0u;
    uu = (uu << 1) | bu;
    vv = (vv << 1) | bv;
  }
  *u = (int32_t)uu;
  *v = (int32_t)vv;
}

// Chung-Lu expected-degree model: each endpoint is drawn with probability
// proportional to its weight, by inverse transform over an integer
// cumulative-weight table cum[0..n) (cum[i] = sum of weights 0..i).
TC_HD int32_t tc_cl_pick(const uint64_t *cum, int64_t n, uint64_t r) {
  const uint64_t total = cum[n - 1];
  const uint64_t x = tc_mulhi(r, total);  // in [0, total)
  int64_t lo = 0, hi = n - 1;              // first index with cum[idx] > x
  while (lo < hi) {
    const int64_t mid = lo + ((hi - lo) >> 1);
    if (cum[mid] > x) hi = mid; else lo = mid + 1;
  }
  return (int32_t)lo;
}

TC_HD void tc_cl_sample(uint64_t key, const uint64_t *cum, int64_t n, uint64_t i, int32_t *u, int32_t *v) {
  *u = tc_cl_pick(cum, n, tc_rand_at(key, 2 * i));
  *v = tc_cl_pick(cum, n, tc_rand_at(key, 2 * i + 1));
}

// Random geometric graph point i: 31-bit integer coordinates in the unit
// square scaled by 2^31, so squared distances fit in uint64 exactly.
TC_HD void tc_rgg_point(uint64_t key, uint64_t i, uint32_t *x, uint32_t *y) {
  *x = (uint32_t)(tc_rand_at(key, 2 * i) >> 33);
  *y = (uint32_t)(tc_rand_at(key, 2 * i + 1) >> 33);
}
