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
// The GB300 decoder stages each block's words in shared memory, parses them
// one group test per loop step through a 64-bit window with both outcomes
// computed by selects (lanes stay converged), and turns the bit planes into
// coefficients with three delta-swap stages over 8-plane chunks (see "Staged
// decoder").
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
// Parse (zfp_parse_planes): one loop step per group-test read.  A step loads
// a 64-bit window at the bit position (three words, two funnel shifts) and
// computes both outcomes with selects: a 1 (the run of zeros after it found
// with one find-first-set, clamped by the bit budget and by coefficient 63,
// decode_ints' two limits) or a 0, which ends the plane and takes the next
// plane's raw bits from the same window.  Only the plane store and the loop
// exit branch, so a warp's lanes stay converged although their blocks take
// different numbers of steps.  A block's leading empty planes (single 0 group
// tests while nothing is significant) are skipped at once.  On the 512^3
// spectral field at rate 2 (about 19 steps per block) this took the full
// decode from 0.390 ms (8-bit group-test table steps, a bit-by-bit tail near
// the limits, branches per outcome) to 0.257 ms; the branching form of the
// same step measured 0.333 ms.
//
// Deposit (zfp_planes_deposit): the plane masks go to a per-thread row of
// shared memory; each 8-plane chunk is read back as 8 rows of 64 bits and all
// eight 8x8 byte columns are transposed at once by three delta-swap stages,
// after which byte g of row k is coefficient 8g + k's bits of those planes.
// ---------------------------------------------------------------------------

// PTX shifts clamp the count: a shift by 32 or more gives 0 (the host
// branch states the same for host builds of this header)
__device__ __forceinline__ uint32_t zfp_shl(uint32_t x, uint32_t s)
{
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm("shl.b32 %0, %1, %2;" : "=r"(r) : "r"(x), "r"(s));
    return r;
#else
    return s >= 32u ? 0u : x << s;
#endif
}
__device__ __forceinline__ uint32_t zfp_shr(uint32_t x, uint32_t s)
{
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm("shr.b32 %0, %1, %2;" : "=r"(r) : "r"(x), "r"(s));
    return r;
#else
    return s >= 32u ? 0u : x >> s;
#endif
}

// decode_ints' bit planes (zfp_decompress.comp:265-294) as masks.  `w`: the
// block's words (LSB first), readable for two words past the block; `pos`:
// the first bit after the header.  Plane r (bit 31 - r of the coefficients)
// goes to pl[2(r - r0)] (coefficients 0..31) and pl[2(r - r0) + 1] (32..63),
// where *r0 is the number of leading empty planes, which are not stored.
// Returns the number of planes decoded, r0 included.
//
// A 64-bit window suffices: a run after a group test needs bits 1..63 (one
// that would reach bit 64 is cut at 63 coefficients first), raw bits after a
// group test number at most 63 (n < 64 there), and 64 raw bits are read only
// where no group test is (n = 64).
__device__ __forceinline__ uint32_t zfp_parse_planes(const uint32_t* w, uint32_t pos, uint32_t budget, uint32_t* pl,
                                                     uint32_t* r0p)
{
    uint32_t bits = budget, n = 0, xlo = 0, xhi = 0, a0, a1;
    a0 = __funnelshift_r(w[pos >> 5], w[(pos >> 5) + 1], pos & 31u);
    const uint32_t r0 = min(a0 ? (uint32_t)__ffs(a0) - 1u : 32u, bits);
    pos += r0;
    bits -= r0;
    *r0p = r0;
    uint32_t r = r0;
    if (r == 32u || bits == 0u) return r;
    pl -= 2u * r0;
    for (;;) {
        const uint32_t i = pos >> 5, sh = pos & 31u;
        const uint32_t w0 = w[i], w1 = w[i + 1], w2 = w[i + 2];
        a0 = __funnelshift_r(w0, w1, sh);
        a1 = __funnelshift_r(w1, w2, sh);
        const uint32_t b0 = __funnelshift_r(a0, a1, 1), b1 = a1 >> 1;  // window bits 1..63
        const bool gtr = n < 64u && bits != 0u;  // a group test is read
        const bool one = gtr && (a0 & 1u);
        // a 1: t zeros before the next one (63: none within the window)
        const uint32_t t = b0 ? (uint32_t)__ffs(b0) - 1u : (b1 ? (uint32_t)__ffs(b1) + 31u : 63u);
        const uint32_t lim = min(63u - n, bits - 1u);
        const uint32_t z = min(t, lim), hit = t < lim ? 1u : 0u;
        const uint32_t nt = n + z;  // the coefficient that becomes significant
        // a 0 (or no read): the plane ends; the next plane's raw bits follow
        const uint32_t o = gtr ? 1u : 0u, be = bits - o, m = min(n, be);
        if (!one) {
            pl[2 * r] = xlo;
            pl[2 * r + 1] = xhi;
            ++r;
            if (r == 32u || be == 0u) break;
        }
        const uint32_t c0 = gtr ? b0 : a0, c1 = gtr ? b1 : a1;
        const uint32_t rlo = c0 & (zfp_shl(1u, m) - 1u), rhi = c1 & zfp_shr(0xffffffffu, 64u - m);
        const uint32_t tlo = xlo | zfp_shl(1u, nt), thi = xhi | zfp_shl(1u, nt - 32u);
        xlo = one ? tlo : rlo;
        xhi = one ? thi : rhi;
        const uint32_t adv = one ? 1u + z + hit : o + m;
        pos += adv;
        bits -= adv;
        n = one ? nt + 1u : n;
    }
    return r;
}

// delta swap: the bits of a at (mask << s) exchange with the bits of b at mask
__device__ __forceinline__ void zfp_dswap(uint32_t& a, uint32_t& b, uint32_t s, uint32_t mask)
{
    const uint32_t t = ((a >> s) ^ b) & mask;
    b ^= t;
    a ^= t << s;
}

// Rows of stored planes 8c .. 8c + 7 (row j = stored plane 8c + 7 - j, zero
// past `np`), transposed: byte g of row k is then coefficient 8g + k's bits
// of those planes, the first at bit 7.
__device__ __forceinline__ void zfp_chunk(const uint32_t* pl, uint32_t c, uint32_t np, uint32_t* L, uint32_t* H)
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 v = reinterpret_cast<const uint4*>(pl + 16u * c)[q];
        const uint32_t p0 = 8u * c + 2u * (uint32_t)q;
        L[7 - 2 * q] = p0 < np ? v.x : 0u;
        H[7 - 2 * q] = p0 < np ? v.y : 0u;
        L[6 - 2 * q] = p0 + 1u < np ? v.z : 0u;
        H[6 - 2 * q] = p0 + 1u < np ? v.w : 0u;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        zfp_dswap(L[j], L[j + 4], 4, 0x0F0F0F0Fu);
        zfp_dswap(H[j], H[j + 4], 4, 0x0F0F0F0Fu);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if ((j & 2) == 0) {
            zfp_dswap(L[j], L[j + 2], 2, 0x33333333u);
            zfp_dswap(H[j], H[j + 2], 2, 0x33333333u);
        }
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
        zfp_dswap(L[j], L[j + 1], 1, 0x55555555u);
        zfp_dswap(H[j], H[j + 1], 1, 0x55555555u);
    }
}

// Coefficients (stream order) from the stored planes r0 .. planes - 1: chunk
// c's byte of a coefficient goes to bits 31 - r0 - 8c down to 24 - r0 - 8c.
__device__ __forceinline__ void zfp_planes_deposit(const uint32_t* pl, uint32_t planes, uint32_t r0, uint32_t* u)
{
    const uint32_t np = planes - r0;
    {
        uint32_t L[8], H[8];
        zfp_chunk(pl, 0u, np, L, H);
        // r0 is 32 only for a block whose 32 planes are all empty: np is 0,
        // every row is zero, and the shift (kept below 32, as C++ requires)
        // moves nothing
        const uint32_t s0 = r0 & 31u;
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                u[8 * g + k] = __byte_perm(L[k], 0u, 0x0444u | ((uint32_t)g << 12)) >> s0;
                u[8 * (g + 4) + k] = __byte_perm(H[k], 0u, 0x0444u | ((uint32_t)g << 12)) >> s0;
            }
    }
    for (uint32_t c = 1; c * 8u < np; ++c) {
        uint32_t L[8], H[8];
        zfp_chunk(pl, c, np, L, H);
        const uint32_t rs = 8u * c + r0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                u[8 * g + k] |= __byte_perm(L[k], 0u, 0x0444u | ((uint32_t)g << 12)) >> rs;
                u[8 * (g + 4) + k] |= __byte_perm(H[k], 0u, 0x0444u | ((uint32_t)g << 12)) >> rs;
            }
    }
}

// One block from its words `w` (2 * rate 32-bit words, 64 * rate bits; staged
// in shared memory, or in place in global memory), readable for two words
// past the block.  `pl` is the thread's plane scratch: 64 words, 16-byte
// aligned (a row of shared memory, or a thread-local array).
__device__ __forceinline__ void zfp_decode_staged(const uint32_t* w, uint32_t max_bits, uint32_t* pl, float* out)
{
    const uint32_t h = w[0];
    if (!(h & 1u)) {
#pragma unroll
        for (int i = 0; i < 64; ++i) out[i] = 0.0f;
        return;
    }
    const int32_t emax = (int32_t)((h >> 1) & 255u) - 127;
    uint32_t r0;
    const uint32_t planes = zfp_parse_planes(w, 9u, max_bits - 9u, pl, &r0);
    uint32_t u[64];
    zfp_planes_deposit(pl, planes, r0, u);
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
// staged words (2 * rate per block, 4 words of padding) and 68 words of plane
// scratch per thread (64 used; 68 keeps the threads' 16-byte rows on
// different banks).  A thread's row also holds its decoded block for the
// warp's coalesced store (zfp_store_warp).
constexpr uint32_t kZfpPlaneWords = 68;
__host__ __device__ __forceinline__ uint32_t zfp_stage_words(uint32_t threads, uint32_t rate)
{
    return threads * 2u * rate + 4u;
}
__host__ __device__ __forceinline__ size_t zfp_stage_smem(uint32_t threads, uint32_t rate)
{
    return ((size_t)zfp_stage_words(threads, rate) + (size_t)threads * kZfpPlaneWords) * 4u;
}
__device__ __forceinline__ uint32_t* zfp_stage_planes(uint32_t* s_words, uint32_t threads, uint32_t rate)
{
    return s_words + zfp_stage_words(threads, rate) + threadIdx.x * kZfpPlaneWords;
}

// The warp's decoded blocks to out[k * 64 ..] for the warp's k-th block,
// k < count, with coalesced 16-byte stores: each thread writes its block into
// its own row (`row`, from zfp_stage_planes), then the warp stores two blocks
// per instruction.  Every lane of the warp calls it (a lane without a block
// passes nothing to write: `v` is not read when has_block is false).
__device__ __forceinline__ void zfp_store_warp(uint32_t* row, const float* v, bool has_block, float* out,
                                               uint32_t count)
{
    if (has_block) {
        float4* r4 = reinterpret_cast<float4*>(row);
#pragma unroll
        for (int i = 0; i < 16; ++i) r4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
    __syncwarp();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t* row0 = row - lane * kZfpPlaneWords;
#pragma unroll
    for (uint32_t k = 0; k < 16; ++k) {
        const uint32_t blk = 2u * k + (lane >> 4);
        if (blk < count)
            reinterpret_cast<float4*>(out + (uint64_t)blk * 64u)[lane & 15u] =
                *reinterpret_cast<const float4*>(row0 + blk * kZfpPlaneWords + 4u * (lane & 15u));
    }
    __syncwarp();
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
