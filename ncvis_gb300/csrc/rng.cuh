// Random streams on the device.
//
// * Pcg64 with O(log n) jump-ahead: the generator the reference seeds per
//   OpenMP thread (src/ncvis.cpp:195, pcg64 from imneme/pcg-cpp).  PCG
//   XSL-RR 128/64 (O'Neill 2014): 128-bit LCG state, seeded as
//   bump(seed + increment), each output rotr64(hi ^ lo, state >> 122) of the
//   freshly bumped state.  Jump-ahead composes the affine LCG step with
//   itself by repeated squaring (F. Brown, "Random number generation with
//   arbitrary strides", Trans. Am. Nucl. Soc. 71, 1994), so every GPU thread
//   can start at its own offset of the one-thread stream.
// * unit_float: std::uniform_real_distribution<float>(0,1) over that stream
//   (generate_canonical<float,24>: one draw scaled by 2^-64, 1.0 clamped to
//   the largest float below it), which the reference uses to initialise Y
//   (src/ncvis.cpp:196-200).
// * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
//   easy as 1, 2, 3", SC'11): the counter-based generator the parallel SGD
//   kernel draws its noise samples from, keyed by the seed and counted by
//   (epoch, edge, sample block).
#pragma once

#include <cstdint>

namespace ncvis_gpu {

typedef unsigned __int128 u128;

struct Pcg64 {
    u128 s;

    __host__ __device__ static u128 mult() {
        return ((u128)2549297995355413924ULL << 64) | 4865540595714422341ULL;
    }
    __host__ __device__ static u128 inc() {
        return ((u128)6364136223846793005ULL << 64) | 1442695040888963407ULL;
    }
    __host__ __device__ explicit Pcg64(uint64_t seed) { s = ((u128)seed + inc()) * mult() + inc(); }

    __host__ __device__ static uint64_t output(u128 st) {
        uint64_t folded = (uint64_t)(st >> 64) ^ (uint64_t)st;
        unsigned rot = (unsigned)(st >> 122);
        return (folded >> rot) | (folded << ((64u - rot) & 63u));
    }
    __host__ __device__ uint64_t next() {
        s = s * mult() + inc();
        return output(s);
    }
    // Advance the state by n steps (n draws) without producing them.
    __host__ __device__ void advance(uint64_t n) {
        u128 acc_mult = 1, acc_plus = 0, cur_mult = mult(), cur_plus = inc();
        while (n) {
            if (n & 1) {
                acc_mult *= cur_mult;
                acc_plus = acc_plus * cur_mult + cur_plus;
            }
            cur_plus = (cur_mult + 1) * cur_plus;
            cur_mult *= cur_mult;
            n >>= 1;
        }
        s = acc_mult * s + acc_plus;
    }
};

__host__ __device__ inline float unit_float(uint64_t draw) {
    float r = (float)draw * 5.42101086242752217e-20f;  // exact scaling by 2^-64
    return r >= 1.0f ? 0.99999994f : r;
}

struct Philox4x32 {
    uint32_t v[4];
};

__host__ __device__ inline void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ inline Philox4x32 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                    uint32_t c3, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c0, hi0, lo0);
        mulhilo32(M1, c2, hi1, lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    Philox4x32 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

// Uniform index in [0, n) from 64 random bits r = hi:lo, floor(r * n / 2^64)
// (multiply-shift; bias <= n/2^64), computed as (hi*n + (lo*n >> 32)) >> 32.
__host__ __device__ inline uint32_t bounded_index(uint32_t lo, uint32_t hi, uint32_t n) {
    const uint64_t a = (uint64_t)hi * n;
    const uint64_t b = ((uint64_t)lo * n) >> 32;
    return (uint32_t)((a + b) >> 32);
}

// Noise sample `s` (0-based) of edge `e` with source `i`, stream tag `tag`
// (the epoch for SGD, a caller-chosen tag for the loss): a uniform index in
// [0, n) other than i.  Philox4x32-10 block (e_lo, e_hi, tag, s/2) under key
// (k0, k1) gives two 64-bit draws, used by even and odd s; an index equal to
// i is redrawn from blocks (e_lo, e_hi ^ retry<<16, tag, s/2 | 2^31) under key
// (k0 ^ retry, k1), at most 64 times, then replaced by i+1 mod n.
__host__ __device__ inline uint32_t noise_index(uint32_t k0, uint32_t k1, uint64_t e, uint32_t tag,
                                                uint32_t s, uint32_t i, uint32_t n) {
    const Philox4x32 r = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), tag, s >> 1, k0, k1);
    const int h = (int)(s & 1);
    uint32_t o = bounded_index(r.v[2 * h], r.v[2 * h + 1], n);
    for (uint32_t retry = 1; o == i; ++retry) {
        if (retry > 64) {
            o = (o + 1 == n) ? 0 : o + 1;
            break;
        }
        const Philox4x32 rr = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32) ^ (retry << 16), tag,
                                            (s >> 1) | 0x80000000u, k0 ^ retry, k1);
        o = bounded_index(rr.v[0], rr.v[1], n);
    }
    return o;
}

// Noise samples 2p and 2p+1 of edge e: the same indices as noise_index for
// those s, from one Philox block.
__host__ __device__ inline void noise_pair(uint32_t k0, uint32_t k1, uint64_t e, uint32_t tag,
                                           uint32_t p, uint32_t i, uint32_t n, uint32_t &o0,
                                           uint32_t &o1) {
    const Philox4x32 r = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), tag, p, k0, k1);
    o0 = bounded_index(r.v[0], r.v[1], n);
    o1 = bounded_index(r.v[2], r.v[3], n);
    if (o0 == i) o0 = noise_index(k0, k1, e, tag, 2 * p, i, n);
    if (o1 == i) o1 = noise_index(k0, k1, e, tag, 2 * p + 1, i, n);
}

// Key words of a 64-bit seed.
__host__ __device__ inline void noise_key(uint64_t seed, uint32_t &k0, uint32_t &k1) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32) ^ 0x5eed1u;
}

}  // namespace ncvis_gpu
