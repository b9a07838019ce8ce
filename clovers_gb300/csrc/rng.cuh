// Counter-based random stream per (pixel, sample) of the render path, shared
// by the wavefront kernels and the guide's sampling kernel.
#pragma once
#include <stdint.h>

namespace clvd {

// Counter-based stream per (pixel, sample): SplitMix64 (Steele et al. 2014)
// output function over key + k*gamma.  Conversions follow rand 0.9:
// f32 = (u32 >> 8) * 2^-24, bool = sign bit.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t key;
  uint32_t counter;
  __device__ void init(uint64_t seed, uint32_t pixel, uint32_t sample) {
    key = mix64(mix64(seed) ^ (((uint64_t)pixel << 32) | (uint64_t)sample));
    counter = 0;
  }
  __device__ __forceinline__ uint32_t u32() {
    ++counter;
    return (uint32_t)(mix64(key + (uint64_t)counter * 0x9E3779B97F4A7C15ull) >> 32);
  }
  __device__ __forceinline__ float f32() { return (float)(u32() >> 8) * 5.9604644775390625e-8f; }
  __device__ __forceinline__ bool boolean() { return (int32_t)u32() < 0; }
  __device__ __forceinline__ float sym() { return 2.0f * f32() - 1.0f; }
};

}  // namespace clvd
