// zfp_device.cuh -- fixed-rate ZFP float32 3-D block codec, device side.
//
// Decoding follows shaders/zfp_decompress.comp:195-384 value for value: a
// 1-bit "block is nonzero" flag, an 8-bit biased common exponent, the embedded
// bit-plane code over 32 planes with group tests (decode_ints, :265-294),
// negabinary to two's complement (:260-263), the ZFP_PERM3D reorder (:101-185),
// the separable inverse lift along z, y, x (:296-354) and the scale by
// 2^(emax-30) (:378-382).  Bit offsets are 64-bit (the reference multiplies
// block_index*max_bits in 32 bits, :199, which wraps past 2^32 bits).
//
// The GB300 decoder works on native 64-bit words: a 64-bit bit buffer instead
// of the emulated {lo,hi} pair, and the unary run of each group test is
// consumed with one find-first-set instead of one bit at a time.
#pragma once

#include <stdint.h>

#include "zfp_perm.inc"

namespace bcmc {

constexpr uint32_t kZfpMaxBitsLimit = 64u * 32u;  // rate <= 32 bits/value

struct BitReader {
    const uint64_t* __restrict__ p;  // next word to fetch
    uint64_t buf;                    // unread bits, LSB first; bits >= n are 0
    uint32_t n;                      // valid bits in buf

    __device__ __forceinline__ void init(const uint64_t* words, uint64_t bit_offset)
    {
        p = words + (bit_offset >> 6);
        const uint32_t s = (uint32_t)(bit_offset & 63u);
        buf = __ldg(p++) >> s;
        n = 64u - s;
    }
    __device__ __forceinline__ void consume(uint32_t c)  // c <= n
    {
        buf = c >= 64u ? 0ull : buf >> c;
        n -= c;
    }
    __device__ __forceinline__ uint32_t bit()
    {
        if (n == 0) {
            buf = __ldg(p++);
            n = 64;
        }
        const uint32_t b = (uint32_t)buf & 1u;
        buf >>= 1;
        --n;
        return b;
    }
    // next k (<= 64) bits of the stream, LSB first
    __device__ __forceinline__ uint64_t bits(uint32_t k)
    {
        if (k == 0) return 0;
        uint64_t v;
        if (k <= n) {
            v = buf;
            consume(k);
        } else {
            const uint64_t w = __ldg(p++);
            v = buf | (w << n);  // n < k <= 64, so n <= 63
            const uint32_t used = k - n;
            buf = used >= 64u ? 0ull : w >> used;
            n = 64u - used;
        }
        return k >= 64u ? v : (v & ((1ull << k) - 1ull));
    }
    // Consume zero bits, at most `limit` of them; if a one comes first it is
    // consumed too and *hit is set.  Returns the zeros consumed.
    __device__ __forceinline__ uint32_t skip_zeros(uint32_t limit, bool* hit)
    {
        uint32_t z = 0;
        *hit = false;
        while (z < limit) {
            if (n == 0) {
                buf = __ldg(p++);
                n = 64;
            }
            const uint32_t rem = limit - z;
            if (buf != 0ull) {
                const uint32_t tz = (uint32_t)__ffsll((long long)buf) - 1u;
                if (tz < rem) {
                    consume(tz + 1u);
                    z += tz;
                    *hit = true;
                    return z;
                }
                consume(rem);
                return z + rem;
            }
            if (n >= rem) {
                consume(rem);
                return z + rem;
            }
            z += n;
            buf = 0;
            n = 0;
        }
        return z;
    }
};

// decode_ints (zfp_decompress.comp:265-294) into u[64] (stream order).
__device__ __forceinline__ void zfp_decode_ints(BitReader& rd, uint32_t budget, uint32_t* u)
{
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = 0;
    uint32_t bits = budget, n = 0;
    for (int k = 31; k >= 0 && bits != 0; --k) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        uint64_t x = rd.bits(m);
        while (n < 64u && bits != 0) {
            --bits;
            if (!rd.bit()) break;
            const uint32_t limit = (63u - (n < 63u ? n : 63u)) < bits ? (63u - (n < 63u ? n : 63u)) : bits;
            bool hit;
            const uint32_t z = rd.skip_zeros(limit, &hit);
            bits -= z + (hit ? 1u : 0u);
            n += z;
            x |= 1ull << n;
            ++n;
        }
        const uint32_t bitk = 1u << k;
        while (x) {
            const int i = __ffsll((long long)x) - 1;
            u[i] |= bitk;
            x &= x - 1ull;
        }
    }
}

// Same decode with the coefficients in registers: each plane is shifted into
// all 64 accumulators (acc = acc*2 + bit), so the critical path is short --
// used where a launch decodes few blocks and latency, not throughput, counts.
__device__ __forceinline__ void zfp_decode_ints_regs(BitReader& rd, uint32_t budget, uint32_t* u)
{
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = 0;
    uint32_t bits = budget, n = 0;
    int k = 31;
    for (; k >= 0 && bits != 0; --k) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        uint64_t x = rd.bits(m);
        while (n < 64u && bits != 0) {
            --bits;
            if (!rd.bit()) break;
            const uint32_t room = 63u - (n < 63u ? n : 63u);
            bool hit;
            const uint32_t z = rd.skip_zeros(room < bits ? room : bits, &hit);
            bits -= z + (hit ? 1u : 0u);
            n += z;
            x |= 1ull << n;
            ++n;
        }
        const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
#pragma unroll
        for (int i = 0; i < 32; ++i) u[i] = (u[i] << 1) | ((lo >> i) & 1u);
#pragma unroll
        for (int i = 0; i < 32; ++i) u[32 + i] = (u[32 + i] << 1) | ((hi >> i) & 1u);
    }
    // planes k..0 were not reached: they are zero
    const uint32_t rest = (uint32_t)(k + 1);
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = rest >= 32u ? 0u : u[i] << rest;
}

__device__ __forceinline__ int32_t zfp_uint2int(uint32_t x)
{
    return (int32_t)((x ^ 0xaaaaaaaau) - 0xaaaaaaaau);
}

// inverse_lift (zfp_decompress.comp:296-332).  WGSL integer arithmetic wraps,
// and streams that are not encoder output (or corrupt ones) do overflow here,
// so adds, subtracts and left shifts run in uint32 (C++ signed overflow would
// be undefined and the compiler may assume it away); only >> is on int32
// (arithmetic shift, as on the reference's int).
__device__ __forceinline__ void zfp_inv_lift(int32_t& x, int32_t& y, int32_t& z, int32_t& w)
{
    uint32_t ux = (uint32_t)x, uy = (uint32_t)y, uz = (uint32_t)z, uw = (uint32_t)w;
    uy += (uint32_t)((int32_t)uw >> 1);
    uw -= (uint32_t)((int32_t)uy >> 1);
    uy += uw;
    uw <<= 1;
    uw -= uy;
    uz += ux;
    ux <<= 1;
    ux -= uz;
    uy += uz;
    uz <<= 1;
    uz -= uy;
    uw += ux;
    ux <<= 1;
    ux -= uw;
    x = (int32_t)ux;
    y = (int32_t)uy;
    z = (int32_t)uz;
    w = (int32_t)uw;
}

__device__ __forceinline__ void zfp_inverse_transform(int32_t* v)
{
#pragma unroll
    for (int i = 0; i < 16; ++i) zfp_inv_lift(v[i], v[i + 16], v[i + 32], v[i + 48]);  // z
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int z = 0; z < 4; ++z) {
            const int b = 16 * z + x;
            zfp_inv_lift(v[b], v[b + 4], v[b + 8], v[b + 12]);  // y
        }
#pragma unroll
    for (int i = 0; i < 16; ++i) zfp_inv_lift(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);  // x
}

// 2^(emax-30) exactly (ldexp(1.f, emax-30), zfp_decompress.comp:378)
__device__ __forceinline__ float zfp_inv_weight(int32_t emax)
{
    const int32_t e = emax - 30;
    if (e >= -126 && e <= 127) return __int_as_float((e + 127) << 23);
    return ldexpf(1.0f, e);
}

// Decode one block starting at `bit_offset` into out[64] (natural order).
// kDeposit: 0 = per-set-bit deposit into a local array, 1 = register
// shift-in per plane (faster on GB300 for both bulk and latency-bound decodes).
template <int kDeposit = 0>
__device__ __forceinline__ void zfp_decode_block(const uint64_t* __restrict__ words,
                                                 uint64_t bit_offset, uint32_t max_bits,
                                                 float* out)
{
    BitReader rd;
    rd.init(words, bit_offset);
    if (!rd.bit()) {
#pragma unroll
        for (int i = 0; i < 64; ++i) out[i] = 0.0f;
        return;
    }
    const int32_t emax = (int32_t)((uint32_t)rd.bits(8) - 127u);
    uint32_t u[64];
    if (kDeposit == 1) zfp_decode_ints_regs(rd, max_bits - 9u, u);
    else zfp_decode_ints(rd, max_bits - 9u, u);
    int32_t v[64];
    uint32_t un[64];
    BCMC_ZFP_GATHER(un, u)
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = zfp_uint2int(un[i]);
    zfp_inverse_transform(v);
    const float w = zfp_inv_weight(emax);
#pragma unroll
    for (int i = 0; i < 64; ++i) out[i] = __fmul_rn(w, __int2float_rn(v[i]));
}

// ---------------------------------------------------------------------------
// Encoder (the reference only decodes): block-floating-point cast, forward
// lift along x, y, z, negabinary reorder and embedded bit-plane coding with
// group tests, per the published fixed-rate ZFP method (Lindstrom 2014).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void zfp_fwd_lift(int32_t& x, int32_t& y, int32_t& z, int32_t& w)
{
    x += w; x >>= 1; w -= x;
    z += y; z >>= 1; y -= z;
    x += z; x >>= 1; z -= x;
    w += y; w >>= 1; y -= w;
    w += y >> 1; y -= w >> 1;
}

struct BitWriter {
    unsigned long long* words;
    uint64_t pos;  // absolute bit position of buf's bit 0
    uint64_t buf;
    uint32_t n;    // bits in buf

    __device__ __forceinline__ void init(unsigned long long* w, uint64_t bit_offset)
    {
        words = w;
        pos = bit_offset & ~63ull;
        n = (uint32_t)(bit_offset & 63u);
        buf = 0;
    }
    __device__ __forceinline__ void flush_word()
    {
        if (buf) atomicOr(words + (pos >> 6), (unsigned long long)buf);
        pos += 64;
        buf = 0;
        n = 0;
    }
    __device__ __forceinline__ uint32_t put_bit(uint32_t b)
    {
        buf |= (uint64_t)(b & 1u) << n;
        if (++n == 64) flush_word();
        return b & 1u;
    }
    // writes the low k (<= 64) bits of v; returns v >> k
    __device__ __forceinline__ uint64_t put_bits(uint64_t v, uint32_t k)
    {
        for (uint32_t i = 0; i < k; ++i) put_bit((uint32_t)(v >> i) & 1u);
        return k >= 64 ? 0ull : v >> k;
    }
    __device__ __forceinline__ void finish()
    {
        if (n) {
            if (buf) atomicOr(words + (pos >> 6), (unsigned long long)buf);
            buf = 0;
            n = 0;
        }
    }
};

__device__ __forceinline__ void zfp_encode_block(const float* f, uint32_t max_bits, BitWriter& bw)
{
    float amax = 0.0f;
#pragma unroll
    for (int i = 0; i < 64; ++i) amax = fmaxf(amax, fabsf(f[i]));
    int emax = -127;
    if (amax > 0.0f) frexpf(amax, &emax);
    const uint32_t e = (uint32_t)(emax + 127);
    if (e == 0) {
        bw.put_bit(0);
        return;
    }
    bw.put_bit(1);
    bw.put_bits(e, 8);
    int32_t v[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = (int32_t)ldexpf(f[i], 30 - emax);
#pragma unroll
    for (int i = 0; i < 16; ++i) zfp_fwd_lift(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);  // x
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int z = 0; z < 4; ++z) {
            const int b = 16 * z + x;
            zfp_fwd_lift(v[b], v[b + 4], v[b + 8], v[b + 12]);  // y
        }
#pragma unroll
    for (int i = 0; i < 16; ++i) zfp_fwd_lift(v[i], v[i + 16], v[i + 32], v[i + 48]);  // z
    uint32_t un[64], u[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) un[i] = ((uint32_t)v[i] + 0xaaaaaaaau) ^ 0xaaaaaaaau;
    BCMC_ZFP_SCATTER(u, un)
    uint32_t bits = max_bits - 9u;
    uint32_t n = 0;
    for (int k = 31; k >= 0 && bits != 0; --k) {
        uint64_t x = 0;
#pragma unroll
        for (int i = 0; i < 64; ++i) x |= (uint64_t)((u[i] >> k) & 1u) << i;
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        x = bw.put_bits(x, m);
        for (; n < 64u && bits != 0 && (bits--, bw.put_bit(x != 0ull)); x >>= 1, n++)
            for (; n < 63u && bits != 0 && (bits--, !bw.put_bit((uint32_t)(x & 1ull))); x >>= 1, n++)
                ;
    }
}

}  // namespace bcmc
