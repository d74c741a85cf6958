// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), written from the
// published round function. Host and device share this code, so every
// synthetic channel is a pure function of (seed, channel index, draw index).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MF_HD __host__ __device__ __forceinline__
#else
#define MF_HD inline
#endif

namespace mfgb {

struct Philox4x32 {
  uint32_t v[4];
};

MF_HD void philox_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = uint64_t(a) * uint64_t(b);
  hi = uint32_t(p >> 32);
  lo = uint32_t(p);
}

MF_HD Philox4x32 philox4x32_10(Philox4x32 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, ctr.v[0], hi0, lo0);
    philox_mulhilo(M1, ctr.v[2], hi1, lo1);
    Philox4x32 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// A per-channel stream: counter = (draw block, channel lo, channel hi, tag).
struct ChannelRng {
  uint32_t k0, k1, c1, c2;
  uint32_t block;
  uint32_t buf[4];
  int left;

  MF_HD ChannelRng(uint64_t seed, uint64_t channel, uint32_t tag)
      : k0(uint32_t(seed)), k1(uint32_t(seed >> 32) ^ tag), c1(uint32_t(channel)), c2(uint32_t(channel >> 32)),
        block(0), left(0) {
    buf[0] = buf[1] = buf[2] = buf[3] = 0;
  }

  MF_HD uint32_t next_u32() {
    if (left == 0) {
      Philox4x32 c;
      c.v[0] = block++;
      c.v[1] = c1;
      c.v[2] = c2;
      c.v[3] = 0x6d66u;  // stream tag "mf"
      const Philox4x32 r = philox4x32_10(c, k0, k1);
      buf[0] = r.v[0];
      buf[1] = r.v[1];
      buf[2] = r.v[2];
      buf[3] = r.v[3];
      left = 4;
    }
    return buf[4 - left--];
  }

  // Uniform double in the open interval (0, 1) from 53 random bits.
  MF_HD double uniform() {
    const uint64_t hi = next_u32(), lo = next_u32();
    const uint64_t x = ((hi << 32) | lo) >> 11;
    return (double(x) + 0.5) * (1.0 / 9007199254740992.0);
  }
};

}  // namespace mfgb
