// Counter-based uniform values of the random density-matrix noise, the same
// function on the host and on the GPU (so every engine draws the same
// wavefunctions for a seed): the splitmix64 output mix (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
// applied to a Weyl-sequence combination of (seed, quantum, element), and
// the top 53 bits scaled to [-1, 1), which every IEEE double machine
// represents exactly.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define BGPU_HD __host__ __device__ __forceinline__
#else
#define BGPU_HD inline
#endif

namespace bgpu {

BGPU_HD double noise_uniform(uint64_t seed, int quantum, int64_t element) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(quantum + 1) + 0xD1B54A32D192ED03ull * (uint64_t)element;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

}  // namespace bgpu
