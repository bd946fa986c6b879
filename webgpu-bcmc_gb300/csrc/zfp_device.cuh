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
// The GB300 decoder stages each block's words in shared memory and reads them
// through a 64-bit window of 32-bit funnel shifts; the group tests are taken 8
// bits per step through a 512-entry state table in shared memory (or a unary
// run per find-first-set where there is no shared memory), and the bit planes
// become coefficients through 8x8 bit transposes (see "Staged decoder").
#pragma once

#include <stdint.h>

#include "zfp_perm.inc"

namespace bcmc {

constexpr uint32_t kZfpMaxBitsLimit = 64u * 32u;  // rate <= 32 bits/value

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

// ---------------------------------------------------------------------------
// Staged decoder: the block's compressed words are first copied into shared
// memory (coalesced loads by the CTA for runs of consecutive blocks, or one
// block per thread), then parsed there.
//
// The parse reads the words through a 32-bit window (a funnel shift of two
// words), takes each plane's raw bits at once and its group tests 8 bits per
// table step (zfp_parse_planes_gt) or one unary run per find-first-set
// (zfp_parse_planes), and writes each plane's 64-bit mask to a per-thread
// scratch; the coefficients are then built from 8-plane chunks with 8x8 bit
// transposes (kDeposit 0) or shifted in plane by plane (kDeposit 1).  On the
// 512^3 spectral field at rate 2 (8 planes, 11 group tests and 72 group-test
// bits per block on average) the table parse takes 268 us against 303 us for
// the find-first-set parse; a parse flattened into one loop of uniform steps
// (raw chunk, table step or single bit, branch-free or not), so that lanes do
// not wait for each other at plane boundaries, measured 296-299 us.
// ---------------------------------------------------------------------------

// Bit window over 32-bit words (LSB first): the 32 bits at the current
// position are one funnel shift of the two words around it.  The window reads
// one word past the last bit it consumes, so a block is followed by at least
// one readable word (staged blocks get padding).
struct ZfpWindow {
    const uint32_t* p;  // next word to load
    uint32_t lo, hi, sh;
    __device__ __forceinline__ void init(const uint32_t* w)
    {
        lo = w[0];
        hi = w[1];
        p = w + 2;
        sh = 0;
    }
    __device__ __forceinline__ uint32_t peek() const { return __funnelshift_r(lo, hi, sh); }
    __device__ __forceinline__ void skip(uint32_t c)  // c <= 32
    {
        sh += c;
        if (sh >= 32u) {
            sh -= 32u;
            lo = hi;
            hi = *p++;
        }
    }
};

__device__ __forceinline__ uint32_t zfp_mask32(uint32_t m) { return m >= 32u ? 0xffffffffu : (1u << m) - 1u; }

// decode_ints' bit planes (zfp_decompress.comp:265-294) as masks: plane 31 - r
// at pl[2r] (coefficients 0..31) and pl[2r + 1] (32..63).  Returns the number
// of planes decoded.  Per plane: the raw bits of the n coefficients already
// significant, then group tests, each a 1 followed by the run of zeros before
// the next significant coefficient (one find-first-set in the common case) or
// a 0 that ends the plane.
__device__ __forceinline__ uint32_t zfp_parse_planes(ZfpWindow& rd, uint32_t budget, uint32_t* pl)
{
    uint32_t bits = budget, n = 0, r = 0;
    for (; r < 32u && bits != 0; ++r) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        uint32_t xlo, xhi = 0;
        if (m <= 32u) {
            xlo = rd.peek() & zfp_mask32(m);
            rd.skip(m);
        } else {
            xlo = rd.peek();
            rd.skip(32);
            xhi = rd.peek() & zfp_mask32(m - 32u);
            rd.skip(m - 32u);
        }
        while (n < 64u && bits != 0) {
            const uint32_t W = rd.peek();
            --bits;
            if (!(W & 1u)) {
                rd.skip(1);
                break;
            }
            const uint32_t limit = min(63u - n, bits);
            const uint32_t Z = W >> 1;
            const uint32_t tz = (uint32_t)__ffs(Z) - 1u;  // 0xffffffff when Z == 0
            uint32_t z;
            if (Z != 0u && tz < limit) {  // the next one is within this window
                rd.skip(tz + 2u);
                bits -= tz + 1u;
                z = tz;
            } else {  // a longer run, or one that reaches the limit
                rd.skip(1);
                z = 0;
                bool hit = false;
                while (z < limit) {
                    const uint32_t V = rd.peek();
                    const uint32_t rem = limit - z;
                    const uint32_t t = (uint32_t)__ffs(V) - 1u;
                    if (V != 0u && t < rem) {
                        rd.skip(t + 1u);
                        z += t;
                        hit = true;
                        break;
                    }
                    const uint32_t step = rem < 32u ? rem : 32u;
                    rd.skip(step);
                    z += step;
                }
                bits -= z + (hit ? 1u : 0u);
            }
            n += z;
            if (n < 32u) xlo |= 1u << n;
            else xhi |= 1u << (n - 32u);
            ++n;
        }
        pl[2 * r] = xlo;
        pl[2 * r + 1] = xhi;
    }
    return r;
}

// Group-test step table.  A plane's group tests read as a two-state machine
// over its bits: in state 0 the next bit is a group test (0 ends the plane,
// 1 enters state 1); in state 1 each bit is the next coefficient's (1: it
// becomes significant, back to state 0).  Entry (state << 8 | b) is what the
// 8 bits b do from `state`, as long as neither the bit budget nor coefficient
// 63 (whose run decode_ints does not read) falls among them:
//   bits 0-3  bits consumed (1..8; fewer when the plane ends)
//   bits 4-7  coefficients passed (0..8)
//   bits 8-15 which of those became significant (bit i: the i-th passed)
//   bit 16    the plane ended
//   bit 17    the state after the last bit consumed
__host__ __device__ constexpr uint32_t zfp_gt_entry(uint32_t idx)
{
    uint32_t s = (idx >> 8) & 1u, dn = 0, mask = 0, c = 0, end = 0;
    while (c < 8u) {
        const uint32_t b = (idx >> c) & 1u;
        ++c;
        if (s == 0u) {
            if (!b) {
                end = 1;
                break;
            }
            s = 1;
        } else {
            if (b) {
                mask |= 1u << dn;
                s = 0;
            }
            ++dn;
        }
    }
    return c | (dn << 4) | (mask << 8) | (end << 16) | (s << 17);
}

constexpr uint32_t kZfpGtWords = 512;
struct ZfpGtTable {
    uint32_t v[kZfpGtWords];
};
constexpr ZfpGtTable zfp_make_gt()
{
    ZfpGtTable t{};
    for (uint32_t i = 0; i < kZfpGtWords; ++i) t.v[i] = zfp_gt_entry(i);
    return t;
}
// built at compile time; a CTA copies it into shared memory (zfp_gt_fill)
static __device__ const ZfpGtTable g_zfp_gt = zfp_make_gt();
static_assert(zfp_make_gt().v[0] == (1u | (1u << 16)), "state 0, bit 0 clear: the plane ends after one bit");
static_assert(zfp_make_gt().v[256] == (8u | (8u << 4) | (1u << 17)), "state 1, eight zeros: a run continues");

// The CTA's threads copy the table into shared memory; the caller
// synchronises before use.
__device__ __forceinline__ void zfp_gt_fill(uint32_t* gt)
{
    for (uint32_t i = threadIdx.x; i < kZfpGtWords; i += blockDim.x) gt[i] = g_zfp_gt.v[i];
}

// zfp_parse_planes with the group tests taken 8 bits per table step: a step
// is taken when it consumes no more bits than the budget has left and passes
// coefficients below 63 only (each of its reads then happens in decode_ints
// too); otherwise, and for the plane's remaining bits, one bit at a time with
// decode_ints' limits (at coefficient 63 or an empty budget a run ends
// without a read and marks the coefficient).
__device__ __forceinline__ uint32_t zfp_parse_planes_gt(ZfpWindow& rd, uint32_t budget, uint32_t* pl,
                                                        const uint32_t* gt)
{
    uint32_t bits = budget, n = 0, r = 0;
    for (; r < 32u && bits != 0; ++r) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        uint64_t x;
        if (m <= 32u) {
            x = rd.peek() & zfp_mask32(m);
            rd.skip(m);
        } else {
            x = rd.peek();
            rd.skip(32);
            x |= (uint64_t)(rd.peek() & zfp_mask32(m - 32u)) << 32;
            rd.skip(m - 32u);
        }
        uint32_t s = 0;
        bool ended = false;
        for (;;) {
            const uint32_t e = gt[(s << 8) | (rd.peek() & 255u)];
            const uint32_t c = e & 15u, dn = (e >> 4) & 15u;
            if (c > bits || n + dn > 63u) break;
            rd.skip(c);
            bits -= c;
            x |= (uint64_t)((e >> 8) & 255u) << n;
            n += dn;
            s = (e >> 17) & 1u;
            if (e & 0x10000u) {
                ended = true;
                break;
            }
        }
        if (!ended) {
            for (;;) {
                if (s == 0u) {
                    if (n >= 64u || bits == 0u) break;
                    --bits;
                    const uint32_t b = rd.peek() & 1u;
                    rd.skip(1);
                    if (!b) break;
                    s = 1;
                } else {
                    if (n < 63u && bits != 0u) {
                        --bits;
                        const uint32_t b = rd.peek() & 1u;
                        rd.skip(1);
                        if (!b) {
                            ++n;
                            continue;
                        }
                    }
                    x |= 1ull << n;
                    ++n;
                    s = 0;
                }
            }
        }
        pl[2 * r] = (uint32_t)x;
        pl[2 * r + 1] = (uint32_t)(x >> 32);
    }
    return r;
}

// 8x8 bit transpose of the 64-bit matrix (hi:lo), row = byte, column = bit
// (three delta swaps)
__device__ __forceinline__ void zfp_transpose8(uint32_t& lo, uint32_t& hi)
{
    uint32_t t;
    t = (lo ^ (lo >> 7)) & 0x00AA00AAu;
    lo ^= t ^ (t << 7);
    t = (hi ^ (hi >> 7)) & 0x00AA00AAu;
    hi ^= t ^ (t << 7);
    t = (lo ^ (lo >> 14)) & 0x0000CCCCu;
    lo ^= t ^ (t << 14);
    t = (hi ^ (hi >> 14)) & 0x0000CCCCu;
    hi ^= t ^ (t << 14);
    t = (lo ^ __funnelshift_r(lo, hi, 28)) & 0xF0F0F0F0u;
    lo ^= t;
    hi ^= t >> 4;
}

// Coefficients (stream order) from the plane masks: each 8-plane chunk is cut
// into eight 8x8 bit matrices (byte g of planes 8c..8c+7), transposed, and
// each result byte is coefficient 8g + i's bits of those planes.
__device__ __forceinline__ void zfp_planes_transposed(const uint32_t* pl, uint32_t planes, uint32_t* u)
{
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = 0;
    for (uint32_t c = 0; c * 8u < planes; ++c) {
        uint32_t w[16];  // planes 8c .. 8c+7: lo, hi
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 v = reinterpret_cast<const uint4*>(pl + 16u * c)[q];
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
            if (8u * c + (uint32_t)r >= planes) w[2 * r] = w[2 * r + 1] = 0u;
        const uint32_t rs = 8u * c;  // bit j of a result byte is plane 24 - 8c + j: (byte << 24) >> 8c
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const int h = g >> 2;
            const uint32_t sb = (uint32_t)(g & 3);
            const uint32_t sel = sb | ((sb + 4u) << 4);
            // matrix byte j = byte g of plane 7 - j (lo word: planes 7..4, hi word: planes 3..0)
            const uint32_t a = __byte_perm(w[14 + h], w[12 + h], sel);
            const uint32_t b = __byte_perm(w[10 + h], w[8 + h], sel);
            const uint32_t d = __byte_perm(w[6 + h], w[4 + h], sel);
            const uint32_t e = __byte_perm(w[2 + h], w[0 + h], sel);
            uint32_t lo = __byte_perm(a, b, 0x5410u), hi = __byte_perm(d, e, 0x5410u);
            zfp_transpose8(lo, hi);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                u[8 * g + i] |= __byte_perm(lo, 0u, 0x0444u | ((uint32_t)i << 12)) >> rs;
                u[8 * g + 4 + i] |= __byte_perm(hi, 0u, 0x0444u | ((uint32_t)i << 12)) >> rs;
            }
        }
    }
}

// The same by shifting each plane into the 64 accumulators.
__device__ __forceinline__ void zfp_planes_shifted(const uint32_t* pl, uint32_t planes, uint32_t* u)
{
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = 0;
    for (uint32_t r = 0; r < planes; ++r) {
        const uint32_t lo = pl[2 * r], hi = pl[2 * r + 1];
#pragma unroll
        for (int i = 0; i < 32; ++i) u[i] = (u[i] << 1) | ((lo >> i) & 1u);
#pragma unroll
        for (int i = 0; i < 32; ++i) u[32 + i] = (u[32 + i] << 1) | ((hi >> i) & 1u);
    }
    const uint32_t rest = 32u - planes;
#pragma unroll
    for (int i = 0; i < 64; ++i) u[i] = rest >= 32u ? 0u : u[i] << rest;
}

// One block from its words `w` (2 * rate 32-bit words, 64 * rate bits; staged
// in shared memory, or in place in global memory), readable for one word past
// the block.  `pl` is the thread's plane scratch: 64 words, 16-byte aligned
// (in shared memory, or a thread-local array).  `gt`: the CTA's group-test
// step table (zfp_gt_fill), or null for the find-first-set parse (decoders
// without shared memory).
template <int kDeposit = 0>
__device__ __forceinline__ void zfp_decode_staged(const uint32_t* w, uint32_t max_bits, uint32_t* pl, float* out,
                                                  const uint32_t* gt = nullptr)
{
    ZfpWindow rd;
    rd.init(w);
    const uint32_t h = rd.peek();
    if (!(h & 1u)) {
#pragma unroll
        for (int i = 0; i < 64; ++i) out[i] = 0.0f;
        return;
    }
    const int32_t emax = (int32_t)((h >> 1) & 255u) - 127;
    rd.skip(9);
    uint32_t u[64];
    const uint32_t planes = gt ? zfp_parse_planes_gt(rd, max_bits - 9u, pl, gt) : zfp_parse_planes(rd, max_bits - 9u, pl);
    if (kDeposit == 0) zfp_planes_transposed(pl, planes, u);
    else zfp_planes_shifted(pl, planes, u);
    int32_t v[64];
    uint32_t un[64];
    BCMC_ZFP_GATHER(un, u)
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = zfp_uint2int(un[i]);
    zfp_inverse_transform(v);
    const float wt = zfp_inv_weight(emax);
#pragma unroll
    for (int i = 0; i < 64; ++i) out[i] = __fmul_rn(wt, __int2float_rn(v[i]));
}

// Shared memory of a staged decode CTA of `threads` threads at `rate`: the
// staged words (2 * rate per block, 4 words of padding), 68 words of plane
// scratch per thread (64 used; 68 keeps the threads' 16-byte rows apart) and
// the group-test step table.
constexpr uint32_t kZfpPlaneWords = 68;
__host__ __device__ __forceinline__ uint32_t zfp_stage_words(uint32_t threads, uint32_t rate)
{
    return threads * 2u * rate + 4u;
}
__host__ __device__ __forceinline__ size_t zfp_stage_smem(uint32_t threads, uint32_t rate)
{
    return ((size_t)zfp_stage_words(threads, rate) + (size_t)threads * kZfpPlaneWords + kZfpGtWords) * 4u;
}
__device__ __forceinline__ uint32_t* zfp_stage_planes(uint32_t* s_words, uint32_t threads, uint32_t rate)
{
    return s_words + zfp_stage_words(threads, rate) + threadIdx.x * kZfpPlaneWords;
}
__device__ __forceinline__ uint32_t* zfp_stage_gt(uint32_t* s_words, uint32_t threads, uint32_t rate)
{
    return s_words + zfp_stage_words(threads, rate) + threads * kZfpPlaneWords;
}

// Copies the words of blocks b0 .. b0+nb-1 (consecutive) to s_words with
// coalesced 8-byte loads, and zeroes the 4 padding words.  All the CTA's
// threads call it; the caller synchronises before reading.
__device__ __forceinline__ void zfp_stage_run(const uint64_t* __restrict__ words, uint64_t b0, uint32_t nb,
                                              uint32_t rate, uint32_t* s_words)
{
    const uint64_t* src = words + b0 * rate;
    uint2* dst = reinterpret_cast<uint2*>(s_words);
    const uint32_t n = nb * rate;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t x = __ldg(src + i);
        dst[i] = make_uint2((uint32_t)x, (uint32_t)(x >> 32));
    }
    if (threadIdx.x < 4) s_words[2u * n + threadIdx.x] = 0u;
}

// Copies the words of block b to this thread's slot of s_words (2 * rate
// words at threadIdx.x * 2 * rate).  The 4 padding words after the last slot
// are zeroed by thread 0; the caller synchronises before any thread reads.
__device__ __forceinline__ void zfp_stage_block(const uint64_t* __restrict__ words, uint64_t b, uint32_t rate,
                                                uint32_t* s_words)
{
    const uint64_t* src = words + b * rate;
    uint2* dst = reinterpret_cast<uint2*>(s_words + threadIdx.x * 2u * rate);
    for (uint32_t i = 0; i < rate; ++i) {
        const uint64_t x = __ldg(src + i);
        dst[i] = make_uint2((uint32_t)x, (uint32_t)(x >> 32));
    }
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
