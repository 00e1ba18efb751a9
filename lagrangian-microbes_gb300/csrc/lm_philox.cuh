// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers:
// As Easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with a Weyl-sequence key
// schedule. Replaces the global MT19937 draws of the reference (interactions.py:20 pair uniform,
// particle_advecter.py:241-242 diffusion kick): a draw is a pure function of (seed, counter), so
// the GPU and the CPU oracle produce identical numbers for identical (seed, step, i, j).
#pragma once
#include <stdint.h>

namespace lm {

constexpr uint32_t PHILOX_M0 = 0xD2511F53u;
constexpr uint32_t PHILOX_M1 = 0xCD9E8D57u;
constexpr uint32_t PHILOX_W0 = 0x9E3779B9u;
constexpr uint32_t PHILOX_W1 = 0xBB67AE85u;

// Stream tags (counter word 3) keep the pair and diffusion streams disjoint.
constexpr uint32_t TAG_PAIR = 0x50414952u;  // "PAIR"
constexpr uint32_t TAG_DIFF = 0x44494646u;  // "DIFF"

struct U4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t lo0 = PHILOX_M0 * c.x, hi0 = __umulhi(PHILOX_M0, c.x);
    uint32_t lo1 = PHILOX_M1 * c.z, hi1 = __umulhi(PHILOX_M1, c.z);
#else
    uint64_t p0 = (uint64_t)PHILOX_M0 * c.x, p1 = (uint64_t)PHILOX_M1 * c.z;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += PHILOX_W0;
    k1 += PHILOX_W1;
  }
  return c;
}

// One Philox block per unordered pair (i < j) at step `step`:
//   u53 = 53-bit uniform integer; the reference's r = np.random.rand() becomes u53 * 2^-53
struct PairDraw { unsigned long long u53; };

__host__ __device__ __forceinline__ PairDraw pair_draw(uint32_t i, uint32_t j, uint32_t step, uint32_t k0,
                                                       uint32_t k1) {
  U4 o = philox4x32_10(U4{i, j, step, TAG_PAIR}, k0, k1);
  PairDraw d;
  d.u53 = ((unsigned long long)o.x << 21) | (o.y >> 11);
  return d;
}

// 64-bit order hash of pair (i < j) at step `step`: the output function of SplitMix64 (Steele, Lea,
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) applied to the pair index
// offset by Weyl multiples of seed and step. A bijection of its 64-bit input, so pairs of one step
// never collide; cheap enough to evaluate for every neighbour-list entry.
__host__ __device__ __forceinline__ unsigned long long order_hash(uint32_t i, uint32_t j, uint32_t step,
                                                                  unsigned long long seed) {
  unsigned long long z = (((unsigned long long)i << 32) | j) + seed * 0x9E3779B97F4A7C15ull +
                         (unsigned long long)step * 0xD1B54A32D192ED03ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Two uniforms in (-1, 1) for the diffusion kick of particle `p` at step `step`
// (first for latitude, second for longitude, the reference's order).
__host__ __device__ __forceinline__ void diffusion_draw(uint32_t p, uint32_t step, uint32_t k0, uint32_t k1,
                                                        float* ulat, float* ulon) {
  U4 o = philox4x32_10(U4{p, step, 0u, TAG_DIFF}, k0, k1);
  // 23-bit uniform at bin centres: (2k+1) * 2^-23 - 1 with k < 2^23 lies in (-1, 1) and every
  // step of it is exact in float32, so CPU and GPU agree bit for bit.
  *ulat = (float)(2u * (o.x >> 9) + 1u) * (1.0f / 8388608.0f) - 1.0f;
  *ulon = (float)(2u * (o.y >> 9) + 1u) * (1.0f / 8388608.0f) - 1.0f;
}

}  // namespace lm
