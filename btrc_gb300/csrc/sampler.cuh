// Per-path samplers.
//   Independent: PCG32 (O'Neill's published pcg32, XSH-RR output, multiplier
//     6364136223846793005) seeded with murmur_hash64A over the pixel coordinates and
//     advanced by sample_index * 65536 (builtin/btrc/builtin/sampler/independent.cpp:11-24,
//     common/btrc/utils/hash.h:12-99). The reference takes PCG from its eDSL's standard
//     library, which is not shipped; the stream constant below is this project's choice.
//   Halton: per-pixel index offset through inverse radical inverses in bases 2 and 3,
//     Owen-scrambled radical inverse per dimension, dimensions start at 2 and wrap at the
//     1000th prime (builtin/btrc/builtin/sampler/halton.cpp:46-116,
//     common/btrc/utils/low_discrepancy.cpp:10-99).
// Everything here is integer or exactly rounded FP32 arithmetic, so host and device
// produce the same bits.
#pragma once

#include <cstdint>

#include "bmath.h"

namespace bt {

constexpr int PRIME_COUNT = 1000;
constexpr uint64_t PCG_MULT = 6364136223846793005ull;
constexpr uint64_t PCG_STREAM = 0xda3e39cb94b95bdbull;
constexpr float ONE_MINUS_EPS = 0x1.fffffep-1f;
constexpr int HALTON_MAX_RES = 128;

struct SamplerState
{
    // independent: a = state, b = inc; halton: a = halton index, b = dimension
    uint64_t a, b;
};

BT_HD uint32_t pcg32_next(uint64_t &state, uint64_t inc)
{
    const uint64_t old = state;
    state = old * PCG_MULT + inc;
    const uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = static_cast<uint32_t>(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
}

BT_HD void pcg32_seed(uint64_t &state, uint64_t &inc, uint64_t initstate, uint64_t initseq)
{
    state = 0u;
    inc = (initseq << 1u) | 1u;
    pcg32_next(state, inc);
    state += initstate;
    pcg32_next(state, inc);
}

// Jump the LCG ahead by delta steps in O(log delta) (Brown, "Random number generation
// with arbitrary strides", 1994).
BT_HD void pcg32_advance(uint64_t &state, uint64_t inc, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
    while(delta > 0)
    {
        if(delta & 1u)
        {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    state = acc_mult * state + acc_plus;
}

BT_HD float pcg32_uniform(uint64_t &state, uint64_t inc)
{
    const float v = static_cast<float>(pcg32_next(state, inc)) * 0x1p-32f;
    return v < ONE_MINUS_EPS ? v : ONE_MINUS_EPS;
}

// murmur_hash64A over 8 bytes (x then y, little endian), seed 0.
BT_HD uint64_t murmur64a_2x32(uint32_t x, uint32_t y)
{
    const uint64_t m = 0xc6a4a7935bd1e995ull;
    const int r = 47;
    uint64_t h = 0ull ^ (8ull * m);
    uint64_t k = static_cast<uint64_t>(x) | (static_cast<uint64_t>(y) << 32);
    k *= m;
    k ^= k >> r;
    k *= m;
    h ^= k;
    h *= m;
    h ^= h >> r;
    h *= m;
    h ^= h >> r;
    return h;
}

BT_HD uint64_t mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7fb5d329728ea185ull;
    v ^= v >> 27;
    v *= 0x81dadef4bc2dd44dull;
    v ^= v >> 33;
    return v;
}

// n / d for n < 2^32 and 2 <= d < 2^32 by one 64x64 high multiply with
// magic = (2^64 - 1) / d + 1 = ceil(2^64 / d): n * magic / 2^64 exceeds n / d by less than
// n / 2^64 < 1 / d, so the floor is exact. magic == 0 divides directly.
BT_HD uint32_t udiv_magic(uint32_t n, uint32_t d, uint64_t magic)
{
#if defined(__CUDA_ARCH__)
    if(magic != 0ull)
        return static_cast<uint32_t>(__umul64hi(static_cast<uint64_t>(n), magic));
#else
    (void)magic;
#endif
    return n / d;
}

BT_HD uint32_t permutation_element(uint32_t i, uint32_t l, uint32_t p, uint64_t magic = 0ull)
{
    uint32_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    do
    {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
    } while(i >= l);
    const uint32_t x = i + p;
    return x - udiv_magic(x, l, magic) * l;
}

BT_HD float owen_scrambled_radical_inverse(uint32_t base, uint64_t a, uint64_t hash, uint64_t magic = 0ull)
{
    const float inv_base = rcp_rn(static_cast<float>(base));
    float inv_base_m = 1.0f;
    uint64_t reversed = 0;
    // digits: loop while 1 - inv_base^m is still distinguishable from 1 in FP32
    while(1.0f - inv_base_m < 1.0f)
    {
        uint64_t next, digit;
        if(a < 0x100000000ull)
        {
            const uint32_t a32 = static_cast<uint32_t>(a);
            next = udiv_magic(a32, base, magic);
            digit = a32 - static_cast<uint32_t>(next) * base;
        }
        else
        {
            next = a / base;
            digit = a - next * base;
        }
        const uint64_t digit_hash = mix_bits(hash ^ reversed);
        digit = permutation_element(static_cast<uint32_t>(digit), base, static_cast<uint32_t>(digit_hash), magic);
        reversed = reversed * base + digit;
        inv_base_m = inv_base_m * inv_base;
        a = next;
    }
    const float v = inv_base_m * static_cast<float>(reversed);
    return v < ONE_MINUS_EPS ? v : ONE_MINUS_EPS;
}

BT_HD uint64_t inverse_radical_inverse(uint64_t inverse, uint32_t base, int digits)
{
    uint64_t index = 0;
    for(int i = 0; i < digits; ++i)
    {
        const uint64_t digit = inverse % base;
        inverse /= base;
        index = index * base + digit;
    }
    return index;
}

// Film-resolution dependent Halton constants (halton.cpp:140-160).
struct HaltonConsts
{
    int32_t scale[2];
    int32_t exponent[2];
    int32_t mult_inverse[2];
    int32_t stride;
    int32_t pad;
};

} // namespace bt
