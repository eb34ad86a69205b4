// ORACLE — test infrastructure, not product code.
//
// The random streams the reference draws from (src/ncvis.cpp:195-200,
// 281-283, 300), restated from their published algorithms because the
// pcg-cpp submodule is absent from the reference checkout:
//   * pcg64 = PCG XSL-RR 128/64 (M. E. O'Neill, 2014) as pcg-cpp's
//     setseq_xsl_rr_128_64: 128-bit LCG, default multiplier and increment,
//     state seeded as bump(seed + increment), each output taken from the
//     freshly bumped state: rotr64(hi ^ lo, state >> 122).
//   * std::uniform_int_distribution<size_t>(0, hi) of GCC 13 libstdc++ on a
//     full 64-bit generator: Lemire's nearly-divisionless method (D. Lemire,
//     ACM TOMACS 29(1), 2019).
//   * std::uniform_real_distribution<float>(0, 1): generate_canonical<float,24>
//     ([rand.util.canonical]): one draw converted to float and scaled by
//     2^-64, with libstdc++'s clamp of 1.0 to the largest float below 1.
#ifndef ORACLE_RNG_H
#define ORACLE_RNG_H

#include <cmath>
#include <cstdint>

namespace orc {

typedef unsigned __int128 u128;

struct Pcg64 {
    u128 s;
    static u128 mult() { return ((u128)2549297995355413924ULL << 64) | 4865540595714422341ULL; }
    static u128 inc() { return ((u128)6364136223846793005ULL << 64) | 1442695040888963407ULL; }
    explicit Pcg64(uint64_t seed) { s = ((u128)seed + inc()) * mult() + inc(); }
    uint64_t operator()() {
        s = s * mult() + inc();
        uint64_t folded = (uint64_t)(s >> 64) ^ (uint64_t)s;
        unsigned rot = (unsigned)(s >> 122);
        return (folded >> rot) | (folded << ((64u - rot) & 63u));
    }
};

// Uniform integer in [0, hi], hi < 2^64 - 1.
inline uint64_t draw_index(Pcg64 &g, uint64_t hi) {
    const uint64_t range = hi + 1;
    u128 prod = (u128)g() * range;
    uint64_t low = (uint64_t)prod;
    if (low < range) {
        const uint64_t floor_mod = (0 - range) % range;
        while (low < floor_mod) {
            prod = (u128)g() * range;
            low = (uint64_t)prod;
        }
    }
    return (uint64_t)(prod >> 64);
}

// Uniform float in [0, 1).
inline float draw_unit(Pcg64 &g) {
    const float scale = 18446744073709551616.0f;  // 2^64
    float r = (float)g() / scale;
    if (r >= 1.0f) r = std::nextafter(1.0f, 0.0f);
    return r;
}

enum Dist { SQUARED_L2 = 0, INNER_PRODUCT = 1, COSINE = 2, CORRELATION = 3 };

}  // namespace orc

#endif
