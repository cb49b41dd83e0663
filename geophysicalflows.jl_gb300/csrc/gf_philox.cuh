// Counter-based random draws (Philox4x32-10) shared by the forcing and the initial-condition
// generators: element e of step `step` uses counter (e, step_lo, step_hi, tag) and key seed,
// so every draw is reproducible and independent of launch shape and device.
#pragma once
#include <cstdint>

#include "gf_fft.cuh"

namespace gf {

// Philox4x32-10 (Salmon et al., SC'11): counter (e, step_lo, step_hi, tag), key = seed.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}
constexpr uint32_t TAG_FORCING = 0x464F5243u;  // counter word 3 of forcing draws
constexpr uint32_t TAG_INITIAL = 0x494E4954u;  // counter word 3 of initial-condition draws

template <class T> __device__ __forceinline__ T u01(uint32_t x) { return (T(x) + T(0.5)) * T(2.3283064365386963e-10); }
__device__ __forceinline__ void sincospi_t(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ void sincospi_t(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ double log_t(double x) { return log(x); }
__device__ __forceinline__ float log_t(float x) { return logf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }

// complex normal with E|z|^2 = 1 (Box-Muller), or a unit random phase
template <class T>
__device__ __forceinline__ cplx<T> draw(uint64_t e, uint64_t step, uint64_t seed, int phase,
                                       uint32_t tag = TAG_FORCING) {
  uint32_t c[4] = {(uint32_t)e, (uint32_t)step, (uint32_t)(step >> 32), tag};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  T s, co;
  if (phase) {
    sincospi_t(T(2) * u01<T>(c[0]), &s, &co);
    return mk<T>(co, s);
  }
  const T r = sqrt_t(T(-2) * log_t(u01<T>(c[0]))) * T(0.70710678118654752440);
  sincospi_t(T(2) * u01<T>(c[1]), &s, &co);
  return mk<T>(r * co, r * s);
}

// df64: the draw is made in FP64 (forcing elements, first stage only) and split
template <>
__device__ __forceinline__ cplx<df64> draw<df64>(uint64_t e, uint64_t step, uint64_t seed, int phase,
                                                 uint32_t tag) {
  const cplx<double> z = draw<double>(e, step, seed, phase, tag);
  return mk<df64>(df64(z.x), df64(z.y));
}

}  // namespace gf
