// jsh_random.h -- counter-based random numbers for the random vector B
// fields (RandomVectorBField and its cell / per-evaluation variants,
// src/BField.cpp:149-193), shared by the host library and the device.
//
// Generator: Philox4x32-10 of Salmon, Moraes, Dror and Shaw, "Parallel
// random numbers: as easy as 1, 2, 3" (SC'11): a 128-bit counter and a 64-bit
// key mapped through ten rounds of two 32x32->64 multiplications with the
// multipliers 0xD2511F53 and 0xCD9E8D57, the key bumped by the Weyl constants
// 0x9E3779B9 and 0xBB67AE85 between rounds.  Integer-only, so every platform
// draws the same bits; the conversions below are exact or correctly
// rounded, so the directions are the same bits on the host and the device.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define JSH_RND_HD __host__ __device__ __forceinline__
#else
#define JSH_RND_HD inline
#endif

struct JshU4 {
  uint32_t x, y, z, w;
};

JSH_RND_HD void jsh_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

JSH_RND_HD JshU4 jsh_philox4x32_10(JshU4 c, uint64_t key) {
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, lo0, hi1, lo1;
    jsh_mulhilo32(0xD2511F53u, c.x, &hi0, &lo0);
    jsh_mulhilo32(0xCD9E8D57u, c.z, &hi1, &lo1);
    c = JshU4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

// Uniform in (0, 1) from 32 bits: (x + 1/2) 2^-32, exact in FP64.
JSH_RND_HD double jsh_u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386962890625e-10; }

// Streams (the counter's high byte): the directions of cells or evaluations,
// and the uniforms of the cell positions.
#define JSH_STREAM_DIRECTION 0x01000000u
#define JSH_STREAM_CELL_POINT 0x02000000u
// k1 of the counters of a cell's direction and of its position uniforms
// (evaluation draws use the frequency index there, always far below them)
#define JSH_CELL_KEY 0xFFFFFFFFu
#define JSH_CELL_POINT_KEY 0xFFFFFFFEu

#if defined(__CUDA_ARCH__)
#define JSH_RND_MUL(a, b) __dmul_rn(a, b)
#define JSH_RND_ADD(a, b) __dadd_rn(a, b)
#define JSH_RND_DIV(a, b) __ddiv_rn(a, b)
#define JSH_RND_SQRT(a) __dsqrt_rn(a)
#else
#define JSH_RND_MUL(a, b) ((a) * (b))
#define JSH_RND_ADD(a, b) ((a) + (b))
#define JSH_RND_DIV(a, b) ((a) / (b))
#define JSH_RND_SQRT(a) sqrt(a)
#endif

// A random unit vector for the counter (k0, k1, k2): points of the cube
// [-1, 1]^3 (coordinates 2U - 1, exact) drawn until one falls in the unit
// ball (attempt a in the counter's low bits), then divided by its norm;
// every operation rounded once, in this order.  64 rejections in a row
// (probability ~ 1e-21) give +z.
JSH_RND_HD void jsh_random_direction(uint64_t seed, uint32_t k0, uint32_t k1, uint32_t k2, double* n) {
  for (uint32_t a = 0; a < 64u; ++a) {
    const JshU4 r = jsh_philox4x32_10(JshU4{k0, k1, k2, JSH_STREAM_DIRECTION | a}, seed);
    const double x = 2.0 * jsh_u01(r.x) - 1.0, y = 2.0 * jsh_u01(r.y) - 1.0, z = 2.0 * jsh_u01(r.z) - 1.0;
    const double r2 = JSH_RND_ADD(JSH_RND_ADD(JSH_RND_MUL(x, x), JSH_RND_MUL(y, y)), JSH_RND_MUL(z, z));
    if (r2 > 0.0 && r2 <= 1.0) {
      const double s = JSH_RND_SQRT(r2);
      n[0] = JSH_RND_DIV(x, s);
      n[1] = JSH_RND_DIV(y, s);
      n[2] = JSH_RND_DIV(z, s);
      return;
    }
  }
  n[0] = 0.0;
  n[1] = 0.0;
  n[2] = 1.0;
}
