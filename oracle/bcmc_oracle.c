/*
 * bcmc_oracle.c -- CPU oracle for the block-compressed marching-cubes path.
 *
 * TEST INFRASTRUCTURE ONLY (see bcmc_oracle.h).  A plain-C restatement of
 * Twinklebear/webgpu-bcmc's compute shaders and their JavaScript orchestration,
 * written to follow the reference's arithmetic exactly:
 *   - WGSL integer semantics: shift counts taken mod 32, wrapping int arithmetic
 *     (built with -fwrapv), arithmetic >> on int;
 *   - f32 arithmetic evaluated in the reference's expression order with no FMA
 *     contraction (built with -ffp-contract=off);
 *   - function-scope arrays zero-initialised, as WGSL does.
 * Parallel loops use OpenMP so the same code is the timed CPU baseline.
 */
#include "bcmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mc_cases.inc"

#define ZFP_BLOCK 64u

int bcmc_oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static uint32_t align_to(uint32_t v, uint32_t a) { return (uint32_t)(((uint64_t)v + a - 1) / a * a); }

/* ZFP_PERM3D (shaders/zfp_decompress.comp:101-185): coefficient i of the
 * embedded stream lives at (x,y,z) = digits of kPermXYZ[i]. */
static const char kPermXYZ[] =
    "000 100 010 001 011 101 110 200 020 002 111 210 201 021 120 102 012 300 030 003 211 "
    "121 112 022 202 220 310 301 031 130 103 013 122 212 221 311 131 113 320 302 032 230 "
    "203 023 222 321 312 132 231 213 123 033 303 330 322 232 223 133 313 331 233 323 332 "
    "333";
static uint32_t g_perm[64];
static int32_t g_tri[256][16];
static uint32_t g_case_count[256];
static int g_tables_ready = 0;

static void init_tables(void)
{
    if (g_tables_ready) return;
    for (int i = 0; i < 64; ++i) {
        const char* t = kPermXYZ + 4 * i;
        g_perm[i] = (uint32_t)(t[0] - '0') + 4u * ((uint32_t)(t[1] - '0') + 4u * (uint32_t)(t[2] - '0'));
    }
    for (int c = 0; c < 256; ++c) {
        const char* s = kOracleCaseEdges[c];
        int n = (int)strlen(s);
        for (int j = 0; j < 16; ++j) g_tri[c][j] = 0;
        for (int j = 0; j < n; ++j) {
            char ch = s[j];
            g_tri[c][j] = (ch >= 'a') ? 10 + (ch - 'a') : (ch - '0');
        }
        g_tri[c][n] = -1;
        g_case_count[c] = (uint32_t)n;
    }
    g_tables_ready = 1;
}

const int32_t* bcmc_oracle_tri_table(void)
{
    init_tables();
    return &g_tri[0][0];
}

/* compute_block_has_vertices.comp:41-51: entries before the -1 terminator */
uint32_t bcmc_oracle_case_vertex_count(uint32_t case_index)
{
    init_tables();
    const int32_t* row = g_tri[case_index & 255u];
    uint32_t n = 0;
    for (uint32_t t = 0; row[t] != -1; ++t) ++n;
    return n;
}

/* ======================================================================== */
/* Emulated uint64 (shaders/zfp_decompress.comp:3-97).  WGSL takes a shift   */
/* count mod 32; wshl/wshr reproduce that for every variable shift.          */
/* ======================================================================== */
typedef struct {
    uint32_t lo, hi;
} emu64;

static inline uint32_t wshl(uint32_t a, uint32_t n) { return a << (n & 31u); }
static inline uint32_t wshr(uint32_t a, uint32_t n) { return a >> (n & 31u); }

static inline emu64 emu_and(emu64 a, emu64 b) { emu64 c = {a.lo & b.lo, a.hi & b.hi}; return c; }
static inline emu64 emu_or(emu64 a, emu64 b) { emu64 c = {a.lo | b.lo, a.hi | b.hi}; return c; }

/* zfp_decompress.comp:49-65 */
static inline emu64 emu_shl(emu64 a, uint32_t n)
{
    if (n == 0) return a;
    emu64 b;
    if (n < 32) {
        const uint32_t carry = a.lo & wshl(0xffffffffu, 32u - n);
        b.lo = wshl(a.lo, n);
        b.hi = wshl(a.hi, n) | wshr(carry, 32u - n);
    } else {
        b.lo = 0;
        b.hi = wshl(a.lo, n - 32u);
    }
    return b;
}

/* zfp_decompress.comp:67-82 */
static inline emu64 emu_shr(emu64 a, uint32_t n)
{
    if (n == 0) return a;
    emu64 b;
    if (n < 32) {
        const uint32_t carry = a.hi & wshr(0xffffffffu, 32u - n);
        b.lo = wshr(a.lo, n) | wshl(carry, 32u - n);
        b.hi = wshr(a.hi, n);
    } else {
        b.lo = wshr(a.hi, n - 32u);
        b.hi = 0;
    }
    return b;
}

/* zfp_decompress.comp:84-97 */
static inline emu64 emu_mask(uint32_t n)
{
    emu64 a = {0, 0};
    if (n > 0 && n < 65) {
        if (n > 32) {
            a.lo = 0xffffffffu;
            a.hi = wshr(0xffffffffu, 64u - n);
        } else {
            a.lo = wshr(0xffffffffu, 32u - n);
            a.hi = 0;
        }
    }
    return a;
}

typedef struct {
    const uint64_t* words;
    uint32_t current_bit;
    uint64_t current_word;
    emu64 buf;
} ereader;

static inline emu64 load_word(const uint64_t* w, uint64_t i)
{
    emu64 r = {(uint32_t)w[i], (uint32_t)(w[i] >> 32)};
    return r;
}

/* zfp_decompress.comp:195-210.  The reference multiplies in 32 bits; the
 * oracle uses 64-bit bit offsets (the zfp semantics) unless asked to wrap. */
static ereader ereader_create(const uint64_t* words, uint64_t block_index, uint32_t max_bits,
                              int emulate_u32_offset)
{
    ereader r;
    r.words = words;
    if (max_bits != 64) {
        if (emulate_u32_offset) {
            const uint32_t off = (uint32_t)block_index * max_bits;
            r.current_word = off / 64u;
            r.current_bit = off % 64u;
        } else {
            const uint64_t off = block_index * (uint64_t)max_bits;
            r.current_word = off / 64u;
            r.current_bit = (uint32_t)(off % 64u);
        }
    } else {
        r.current_word = emulate_u32_offset ? (uint32_t)block_index : block_index;
        r.current_bit = 0;
    }
    r.buf = load_word(words, r.current_word);
    r.buf = emu_shr(r.buf, r.current_bit);
    return r;
}

/* zfp_decompress.comp:212-217 */
static inline void ereader_advance(ereader* r)
{
    r->current_bit = 0;
    ++r->current_word;
    r->buf = load_word(r->words, r->current_word);
}

/* zfp_decompress.comp:219-230 */
static inline uint32_t ereader_bit(ereader* r)
{
    const uint32_t bit = r->buf.lo & 1u;
    ++r->current_bit;
    r->buf = emu_shr(r->buf, 1);
    if (r->current_bit >= 64) ereader_advance(r);
    return bit;
}

/* zfp_decompress.comp:233-257 */
static inline emu64 ereader_bits(ereader* r, uint32_t n_bits)
{
    const uint32_t rem_bits = 64u - r->current_bit;
    const uint32_t first_read = rem_bits < n_bits ? rem_bits : n_bits;
    emu64 mask = emu_mask(first_read);
    emu64 bits = emu_and(r->buf, mask);
    r->buf = emu_shr(r->buf, n_bits);
    r->current_bit += first_read;
    uint32_t next_read = 0;
    if (n_bits >= rem_bits) {
        ereader_advance(r);
        next_read = n_bits - first_read;
    }
    mask = emu_mask(next_read);
    bits = emu_or(bits, emu_shl(emu_and(r->buf, mask), first_read));
    r->buf = emu_shr(r->buf, next_read);
    r->current_bit += next_read;
    return bits;
}

/* zfp_decompress.comp:260-263 */
static inline int32_t uint2int(uint32_t x) { return (int32_t)((x ^ 0xaaaaaaaau) - 0xaaaaaaaau); }

/* zfp_decompress.comp:265-294 */
static void decode_ints_emu(ereader* r, uint32_t block_max_bits, uint32_t block[64])
{
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) block[i] = 0;
    const emu64 one = {1u, 0u};
    emu64 x = {0, 0};
    uint32_t bits = block_max_bits;
    for (uint32_t k = 32, n = 0; bits != 0 && k-- > 0;) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        x = ereader_bits(r, m);
        for (; n < ZFP_BLOCK && bits != 0 && (bits--, ereader_bit(r) != 0); x = emu_or(x, emu_shl(one, n++))) {
            for (; n < ZFP_BLOCK - 1 && bits != 0 && (bits--, ereader_bit(r) == 0); ++n)
                ;
        }
        for (uint32_t i = 0; i < ZFP_BLOCK; ++i, x = emu_shr(x, 1)) block[i] += (x.lo & 1u) << k;
    }
}

/* ---- native 64-bit reader: same bits, no emulation ---------------------- */
typedef struct {
    const uint64_t* words;
    uint64_t pos; /* absolute bit position */
} nreader;

static inline uint64_t nread(nreader* r, uint32_t n)
{
    if (n == 0) return 0;
    const uint64_t wi = r->pos >> 6;
    const uint32_t b = (uint32_t)(r->pos & 63u);
    uint64_t v = r->words[wi] >> b;
    if (b != 0 && b + n > 64) v |= r->words[wi + 1] << (64u - b);
    if (n < 64) v &= (((uint64_t)1) << n) - 1u;
    r->pos += n;
    return v;
}

static void decode_ints_native(nreader* r, uint32_t block_max_bits, uint32_t block[64])
{
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) block[i] = 0;
    uint32_t bits = block_max_bits;
    for (uint32_t k = 32, n = 0; bits != 0 && k-- > 0;) {
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        uint64_t x = nread(r, m);
        for (; n < 64 && bits != 0 && (bits--, nread(r, 1) != 0); x |= ((uint64_t)1) << n++) {
            for (; n < 63 && bits != 0 && (bits--, nread(r, 1) == 0); ++n)
                ;
        }
        for (uint32_t i = 0; i < 64; ++i, x >>= 1) block[i] += (uint32_t)(x & 1u) << k;
    }
}

/* zfp_decompress.comp:296-332 */
static inline void inverse_lift(int32_t* b, uint32_t s, uint32_t idx)
{
    int32_t x = b[idx], y = b[idx + s], z = b[idx + 2 * s], w = b[idx + 3 * s];
    y += w >> 1;
    w -= y >> 1;
    y += w;
    w = (int32_t)((uint32_t)w << 1);
    w -= y;
    z += x;
    x = (int32_t)((uint32_t)x << 1);
    x -= z;
    y += z;
    z = (int32_t)((uint32_t)z << 1);
    z -= y;
    w += x;
    x = (int32_t)((uint32_t)x << 1);
    x -= w;
    b[idx] = x;
    b[idx + s] = y;
    b[idx + 2 * s] = z;
    b[idx + 3 * s] = w;
}

/* zfp_decompress.comp:334-354 */
static void inverse_transform(int32_t* b)
{
    for (uint32_t y = 0; y < 4; ++y)
        for (uint32_t x = 0; x < 4; ++x) inverse_lift(b, 16, x + 4 * y);
    for (uint32_t x = 0; x < 4; ++x)
        for (uint32_t z = 0; z < 4; ++z) inverse_lift(b, 4, 16 * z + x);
    for (uint32_t z = 0; z < 4; ++z)
        for (uint32_t y = 0; y < 4; ++y) inverse_lift(b, 1, 4 * y + 16 * z);
}

/* zfp_decompress.comp:356-384, after the header has been read */
static void finish_block(const uint32_t ublock[64], int32_t emax, float out[64])
{
    int32_t iblock[64];
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) iblock[g_perm[i]] = uint2int(ublock[i]);
    inverse_transform(iblock);
    const float inv_w = ldexpf(1.0f, emax - 30);
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) out[i] = inv_w * (float)iblock[i];
}

void bcmc_oracle_decode_block(const uint64_t* words, uint64_t block_index, uint32_t max_bits,
                              int emulate_u32_offset, float out[64])
{
    init_tables();
    ereader r = ereader_create(words, block_index, max_bits, emulate_u32_offset);
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) out[i] = 0.0f; /* WGSL zero-init */
    const uint32_t s_cont = ereader_bit(&r);
    if (s_cont != 0) {
        const int32_t emax = (int32_t)(ereader_bits(&r, 8).lo - 127u);
        uint32_t ublock[64];
        decode_ints_emu(&r, max_bits - 9u, ublock);
        finish_block(ublock, emax, out);
    }
}

void bcmc_oracle_decode_block_ints(const uint64_t* words, uint64_t block_index, uint32_t max_bits,
                                   uint32_t out[64], uint32_t* s_cont, int32_t* emax)
{
    init_tables();
    ereader r = ereader_create(words, block_index, max_bits, 0);
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) out[i] = 0;
    *s_cont = ereader_bit(&r);
    *emax = 0;
    if (*s_cont != 0) {
        *emax = (int32_t)(ereader_bits(&r, 8).lo - 127u);
        decode_ints_emu(&r, max_bits - 9u, out);
    }
}

void bcmc_oracle_decode_block_native(const uint64_t* words, uint64_t block_index,
                                     uint32_t max_bits, float out[64])
{
    init_tables();
    nreader r = {words, block_index * (uint64_t)max_bits};
    for (uint32_t i = 0; i < ZFP_BLOCK; ++i) out[i] = 0.0f;
    if (nread(&r, 1) != 0) {
        const int32_t emax = (int32_t)((uint32_t)nread(&r, 8) - 127u);
        uint32_t ublock[64];
        decode_ints_native(&r, max_bits - 9u, ublock);
        finish_block(ublock, emax, out);
    }
}

void bcmc_oracle_decode_volume(const uint64_t* words, uint64_t nblocks, uint32_t max_bits,
                               float* out)
{
    init_tables();
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblocks; ++b)
        bcmc_oracle_decode_block(words, (uint64_t)b, max_bits, 0, out + (uint64_t)b * 64u);
}

/* ======================================================================== */
/* ZFP fixed-rate encoder, written from the published method (Lindstrom     */
/* 2014): block-floating-point cast, forward decorrelating lift, negabinary */
/* reorder, embedded bit-plane coding with group tests, zero padding to the */
/* fixed per-block budget.  Partial blocks are padded the way zfp pads them. */
/* ======================================================================== */
uint64_t bcmc_oracle_stream_words(const uint32_t dims[3], uint32_t max_bits)
{
    const uint64_t nb = (uint64_t)(align_to(dims[0], 4) / 4) * (align_to(dims[1], 4) / 4) *
                        (align_to(dims[2], 4) / 4);
    return (nb * max_bits + 63u) / 64u + 1u;
}

typedef struct {
    uint64_t* words;
    uint64_t pos;
} bwriter;

static inline uint32_t bw_bit(bwriter* w, uint32_t bit)
{
    if (bit) w->words[w->pos >> 6] |= ((uint64_t)1) << (w->pos & 63u);
    ++w->pos;
    return bit;
}

/* writes the low n bits of v, returns v >> n */
static inline uint64_t bw_bits(bwriter* w, uint64_t v, uint32_t n)
{
    for (uint32_t i = 0; i < n; ++i) bw_bit(w, (uint32_t)((v >> i) & 1u));
    return n >= 64 ? 0 : v >> n;
}

/* pad a partial row of n valid samples at stride s (zfp's pad rule) */
static void pad_row(float* p, uint32_t n, uint32_t s)
{
    switch (n) {
    case 0: p[0] = 0.0f; /* fall through */
    case 1: p[1 * s] = p[0]; /* fall through */
    case 2: p[2 * s] = p[1 * s]; /* fall through */
    case 3: p[3 * s] = p[0]; /* fall through */
    default: break;
    }
}

static inline void forward_lift(int32_t* p, uint32_t s)
{
    int32_t x = p[0], y = p[s], z = p[2 * s], w = p[3 * s];
    x += w; x >>= 1; w -= x;
    z += y; z >>= 1; y -= z;
    x += z; x >>= 1; z -= x;
    w += y; w >>= 1; y -= w;
    w += y >> 1; y -= w >> 1;
    p[0] = x; p[s] = y; p[2 * s] = z; p[3 * s] = w;
}

static void encode_block(const float fblock[64], uint32_t max_bits, bwriter* w)
{
    float amax = 0.0f;
    for (int i = 0; i < 64; ++i) {
        const float a = fabsf(fblock[i]);
        if (a > amax) amax = a;
    }
    int emax = -127;
    if (amax > 0.0f) frexpf(amax, &emax);
    const uint32_t e = (uint32_t)(emax + 127);
    if (e == 0) {
        bw_bit(w, 0); /* all-zero block: one 0 bit, rest is padding */
        return;
    }
    bw_bit(w, 1);
    bw_bits(w, e, 8);
    int32_t iblock[64];
    const double s = ldexp(1.0, 30 - emax);
    for (int i = 0; i < 64; ++i) iblock[i] = (int32_t)(s * (double)fblock[i]);
    for (uint32_t z = 0; z < 4; ++z)
        for (uint32_t y = 0; y < 4; ++y) forward_lift(iblock + 4 * y + 16 * z, 1);
    for (uint32_t x = 0; x < 4; ++x)
        for (uint32_t z = 0; z < 4; ++z) forward_lift(iblock + 16 * z + x, 4);
    for (uint32_t y = 0; y < 4; ++y)
        for (uint32_t x = 0; x < 4; ++x) forward_lift(iblock + x + 4 * y, 16);
    uint32_t ublock[64];
    for (int i = 0; i < 64; ++i) ublock[i] = ((uint32_t)iblock[g_perm[i]] + 0xaaaaaaaau) ^ 0xaaaaaaaau;
    uint32_t bits = max_bits - 9u;
    for (uint32_t k = 32, n = 0; bits != 0 && k-- > 0;) {
        uint64_t x = 0;
        for (uint32_t i = 0; i < 64; ++i) x += (uint64_t)((ublock[i] >> k) & 1u) << i;
        const uint32_t m = n < bits ? n : bits;
        bits -= m;
        x = bw_bits(w, x, m);
        for (; n < 64 && bits != 0 && (bits--, bw_bit(w, x != 0)); x >>= 1, n++)
            for (; n < 63 && bits != 0 && (bits--, !bw_bit(w, (uint32_t)(x & 1u))); x >>= 1, n++)
                ;
    }
}

int bcmc_oracle_zfp_encode(const float* field, const uint32_t dims[3], uint32_t max_bits,
                           uint64_t* words)
{
    if (max_bits < 10) return -1;
    init_tables();
    const uint32_t nbx = align_to(dims[0], 4) / 4, nby = align_to(dims[1], 4) / 4,
                   nbz = align_to(dims[2], 4) / 4;
    const uint64_t nblocks = (uint64_t)nbx * nby * nbz;
    memset(words, 0, bcmc_oracle_stream_words(dims, max_bits) * sizeof(uint64_t));
    /* Blocks whose bit range shares a word with a neighbour are written
     * serially; with max_bits a multiple of 64 every block owns its words. */
    const int shared_words = (max_bits % 64u) != 0;
#pragma omp parallel for schedule(static) if (!shared_words)
    for (int64_t bi = 0; bi < (int64_t)nblocks; ++bi) {
        const uint64_t b = (uint64_t)bi;
        const uint32_t bx = (uint32_t)(b % nbx), by = (uint32_t)((b / nbx) % nby),
                       bz = (uint32_t)(b / ((uint64_t)nbx * nby));
        const uint32_t x0 = 4 * bx, y0 = 4 * by, z0 = 4 * bz;
        const uint32_t nx = dims[0] - x0 < 4 ? dims[0] - x0 : 4;
        const uint32_t ny = dims[1] - y0 < 4 ? dims[1] - y0 : 4;
        const uint32_t nz = dims[2] - z0 < 4 ? dims[2] - z0 : 4;
        float blk[64];
        for (uint32_t z = 0; z < nz; ++z) {
            for (uint32_t y = 0; y < ny; ++y) {
                for (uint32_t x = 0; x < nx; ++x)
                    blk[16 * z + 4 * y + x] =
                        field[(uint64_t)(x0 + x) +
                              (uint64_t)dims[0] * ((uint64_t)(y0 + y) + (uint64_t)dims[1] * (z0 + z))];
                pad_row(blk + 16 * z + 4 * y, nx, 1);
            }
            for (uint32_t x = 0; x < 4; ++x) pad_row(blk + 16 * z + x, ny, 4);
        }
        for (uint32_t y = 0; y < 4; ++y)
            for (uint32_t x = 0; x < 4; ++x) pad_row(blk + 4 * y + x, nz, 16);
        bwriter w = {words, b * (uint64_t)max_bits};
        encode_block(blk, max_bits, &w);
    }
    return 0;
}

/* ======================================================================== */
/* zfp_compute_block_range.comp:19-61                                        */
/* ======================================================================== */
static inline float glsl_min(float x, float y) { return y < x ? y : x; }
static inline float glsl_max(float x, float y) { return x < y ? y : x; }

void bcmc_oracle_block_ranges(const uint64_t* words, const uint32_t dims[3], uint32_t max_bits,
                              float* ranges)
{
    init_tables();
    const uint32_t nbx = align_to(dims[0], 4) / 4, nby = align_to(dims[1], 4) / 4,
                   nbz = align_to(dims[2], 4) / 4;
    const uint64_t nblocks = (uint64_t)nbx * nby * nbz;
    /* total_blocks = (padded_dims.x * padded_dims.y) / 64 * padded_dims.z in
     * u32 (zfp_compute_block_range.comp:22): the division truncates when
     * nbx*nby is not a multiple of 4, and blocks from there on keep the zero
     * the freshly created range buffer holds (compressed_marching_cubes.js:526-529). */
    const uint32_t ranged = (align_to(dims[0], 4) * align_to(dims[1], 4)) / 64u * align_to(dims[2], 4);
#pragma omp parallel for schedule(static)
    for (int64_t bi = 0; bi < (int64_t)nblocks; ++bi) {
        const uint64_t b = (uint64_t)bi;
        if (b >= ranged) {
            ranges[2 * b] = 0.0f;
            ranges[2 * b + 1] = 0.0f;
            continue;
        }
        float blk[64];
        bcmc_oracle_decode_block(words, b, max_bits, 0, blk);
        const uint32_t x0 = (uint32_t)(b % nbx) * 4, y0 = (uint32_t)((b / nbx) % nby) * 4,
                       z0 = (uint32_t)(b / ((uint64_t)nbx * nby)) * 4;
        const uint32_t px = (x0 + 4 > dims[0]) ? dims[0] - x0 : 4;
        const uint32_t py = (y0 + 4 > dims[1]) ? dims[1] - y0 : 4;
        const uint32_t pz = (z0 + 4 > dims[2]) ? dims[2] - z0 : 4;
        float lo = 1e20f, hi = -1e20f;
        for (uint32_t z = 0; z < pz; ++z)
            for (uint32_t y = 0; y < py; ++y)
                for (uint32_t x = 0; x < px; ++x) {
                    lo = glsl_min(lo, blk[16 * z + 4 * y + x]);
                    hi = glsl_max(hi, blk[16 * z + 4 * y + x]);
                }
        ranges[2 * b] = lo;
        ranges[2 * b + 1] = hi;
    }
}

/* ======================================================================== */
/* mc_isosurface.vert:51-60 with block_vertex_position.comp:19-26             */
/* ======================================================================== */
void bcmc_oracle_unpack_vertices(const uint32_t* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                                 const float* proj_view, float* world, float* clip)
{
    const uint32_t nbx = align_to(dims[0], 4) / 4, nby = align_to(dims[1], 4) / 4;
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t c = verts[2 * i], id = verts[2 * i + 1];
        const uint32_t b[3] = {id % nbx, (id / nbx) % nby, id / (nbx * nby)};
        const float q[3] = {(float)((c & 0x3ff00000u) >> 20), (float)((c & 0x000ffc00u) >> 10),
                            (float)(c & 0x000003ffu)};
        float w[3];
        for (int k = 0; k < 3; ++k) {
            const float d = (q[k] * 4.0f) / 1023.0f + 0.5f; /* decompress_position */
            const float wp = 4.0f * (float)b[k] + d;
            w[k] = (scale ? scale[k] : 1.0f) * (wp / (float)dims[k] - 0.5f);
            world[3 * i + k] = w[k];
        }
        if (proj_view && clip) {
            for (int r = 0; r < 4; ++r) {
                float acc = proj_view[r] * w[0];
                acc = acc + proj_view[4 + r] * w[1];
                acc = acc + proj_view[8 + r] * w[2];
                acc = acc + proj_view[12 + r] * 1.0f;
                clip[4 * i + r] = acc;
            }
        }
    }
}

/* ======================================================================== */
/* The render pass (js/bcmc.js:174-190,237-265,377-391;                      */
/* shaders/mc_isosurface.vert:35-60, mc_isosurface.frag:15-40), headless.    */
/* Rasterisation follows the WebGPU rules the reference relies on: pixel     */
/* centres at +0.5, NDC y up with row 0 at the top, depth = NDC z in [0, 1], */
/* "less" against 1.0, 1/256-pixel snapping, top-left rule; ties at equal    */
/* depth go to the earlier triangle.  Each f32 step is one rounded operation */
/* in the order the CUDA kernels use and the edge functions are exact        */
/* integers, so the depth and triangle buffers are reproduced bit for bit.   */
/* ======================================================================== */
typedef struct {
    float x, y, z;
} ov3;

static ov3 ov3_sub(ov3 a, ov3 b) { return (ov3){a.x - b.x, a.y - b.y, a.z - b.z}; }
static float ov3_dot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static ov3 ov3_scale(ov3 a, float s) { return (ov3){a.x * s, a.y * s, a.z * s}; }
static ov3 ov3_norm(ov3 a) /* GLSL normalize: x / length(x) */
{
    const float len = sqrtf(ov3_dot(a, a));
    return (ov3){a.x / len, a.y / len, a.z / len};
}
static ov3 ov3_cross(ov3 a, ov3 b)
{
    return (ov3){a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static float g_min(float x, float y) { return y < x ? y : x; } /* GLSL min */
static float g_max(float x, float y) { return x < y ? y : x; } /* GLSL max */
static float g_clamp01(float x) { return g_min(g_max(x, 0.0f), 1.0f); }

void bcmc_oracle_fog_enter(const float* world, uint64_t n, const float eye[3], const float scale[3], float* tenter)
{
    const float o[3] = {eye[0], eye[1], eye[2]};
    float hh[3];
    for (int k = 0; k < 3; ++k) hh[k] = (scale ? scale[k] : 1.0f) * 0.5f;
    for (uint64_t i = 0; i < n; ++i) {
        const ov3 d = ov3_norm(ov3_sub((ov3){world[3 * i], world[3 * i + 1], world[3 * i + 2]}, (ov3){o[0], o[1], o[2]}));
        const float dd[3] = {d.x, d.y, d.z};
        float tmin[3];
        for (int k = 0; k < 3; ++k) {
            const float inv = 1.0f / dd[k];
            const float ta = (-hh[k] - o[k]) * inv, tb = (hh[k] - o[k]) * inv;
            tmin[k] = g_min(ta, tb);
        }
        tenter[i] = g_max(g_max(tmin[0], g_max(tmin[1], tmin[2])), 0.0f);
    }
}

/* Screen positions snapped to 1/256 pixel, edge functions in exact 64-bit
 * integers (watertight with the top-left rule). */
typedef struct {
    int x[3], y[3];
    float z[3];
    int idx[3];
    long long area;
} otri;

static long long edge_fn(int ax, int ay, int bx, int by, int px, int py)
{
    return (long long)(bx - ax) * (long long)(py - ay) - (long long)(by - ay) * (long long)(px - ax);
}
static int top_left(int ax, int ay, int bx, int by) { return (ay == by && bx > ax) || (by < ay); }
static int floor_div256(int v) { return v >= 0 ? v / 256 : -((255 - v) / 256); }

/* 0 when the triangle is not drawn (w <= 1e-6, beyond +-2^21 pixels, not
 * finite, zero area) */
static int tri_setup(const float* c, uint32_t w, uint32_t h, otri* t)
{
    for (int k = 0; k < 3; ++k) {
        const float cw = c[4 * k + 3];
        if (!(cw > 1e-6f)) return 0;
        const float nx = c[4 * k] / cw, ny = c[4 * k + 1] / cw;
        const float sx = (nx * 0.5f + 0.5f) * (float)w, sy = (0.5f - ny * 0.5f) * (float)h;
        if (!(fabsf(sx) <= 2097152.0f && fabsf(sy) <= 2097152.0f)) return 0;
        t->x[k] = (int)rintf(sx * 256.0f);
        t->y[k] = (int)rintf(sy * 256.0f);
        t->z[k] = c[4 * k + 2] / cw;
        t->idx[k] = k;
    }
    t->area = edge_fn(t->x[0], t->y[0], t->x[1], t->y[1], t->x[2], t->y[2]);
    if (t->area == 0) return 0;
    if (t->area < 0) {
        int tmp = t->x[1];
        t->x[1] = t->x[2];
        t->x[2] = tmp;
        tmp = t->y[1];
        t->y[1] = t->y[2];
        t->y[2] = tmp;
        const float tz = t->z[1];
        t->z[1] = t->z[2];
        t->z[2] = tz;
        t->idx[1] = 2;
        t->idx[2] = 1;
        t->area = -t->area;
    }
    return 1;
}

static void edges_at(const otri* t, int px, int py, long long e[3])
{
    const int cx = px * 256 + 128, cy = py * 256 + 128;
    e[0] = edge_fn(t->x[1], t->y[1], t->x[2], t->y[2], cx, cy);
    e[1] = edge_fn(t->x[2], t->y[2], t->x[0], t->y[0], cx, cy);
    e[2] = edge_fn(t->x[0], t->y[0], t->x[1], t->y[1], cx, cy);
}

/* mc_isosurface.frag:15-40 for one fragment: world position, interpolated
 * t_enter, the triangle's three world vertices (flat normal from its edges,
 * which the frag's screen derivatives span), fog on/off -> rgba. */
void bcmc_oracle_shade(const float wp3[3], float te, const float eye[3], const float* tri_world, int fog,
                       float out[4])
{
    const ov3 wp = {wp3[0], wp3[1], wp3[2]};
    ov3 v = ov3_sub(wp, (ov3){eye[0], eye[1], eye[2]});
    const float dist = sqrtf(ov3_dot(v, v));
    v = ov3_scale(ov3_norm(v), -1.0f);
    const ov3 light = v;
    const ov3 w0 = {tri_world[0], tri_world[1], tri_world[2]}, w1 = {tri_world[3], tri_world[4], tri_world[5]},
              w2 = {tri_world[6], tri_world[7], tri_world[8]};
    ov3 nrm = ov3_norm(ov3_cross(ov3_sub(w1, w0), ov3_sub(w2, w0)));
    if (ov3_dot(nrm, light) < 0.0f) nrm = ov3_scale(nrm, -1.0f);
    const float base[3] = {0.3f, 0.3f, 0.9f};
    const ov3 hv = ov3_norm((ov3){v.x + light.x, v.y + light.y, v.z + light.z});
    const float diff = 0.6f * g_clamp01(ov3_dot(light, nrm));
    const float spec = 0.1f * powf(g_clamp01(ov3_dot(nrm, hv)), 5.0f);
    float col[3];
    for (int k = 0; k < 3; ++k) col[k] = (base[k] * 0.2f + diff * base[k]) + spec;
    if (fog) {
        const float f = expf(-1.0f * g_max(dist - (te + 0.1f), 0.0f));
        for (int k = 0; k < 3; ++k) col[k] = f * col[k] + (1.0f - f);
    }
    out[0] = col[0];
    out[1] = col[1];
    out[2] = col[2];
    out[3] = 1.0f;
}

int bcmc_oracle_render(const uint32_t* verts, uint64_t n, const uint32_t dims[3], const float scale[3],
                       const float proj_view[16], const float eye[3], int fog, uint32_t width, uint32_t height,
                       float* rgba, float* depth, uint32_t* triangle)
{
    const uint64_t ntri = n / 3, nv = ntri * 3, npix = (uint64_t)width * height;
    float* world = (float*)malloc((nv ? nv : 1) * 3 * sizeof(float));
    float* clip = (float*)malloc((nv ? nv : 1) * 4 * sizeof(float));
    float* tenter = (float*)malloc((nv ? nv : 1) * sizeof(float));
    uint64_t* keys = (uint64_t*)malloc((npix ? npix : 1) * sizeof(uint64_t));
    if (!world || !clip || !tenter || !keys) {
        free(world);
        free(clip);
        free(tenter);
        free(keys);
        return -1;
    }
    bcmc_oracle_unpack_vertices(verts, nv, dims, scale, proj_view, world, clip);
    if (fog) bcmc_oracle_fog_enter(world, nv, eye, scale, tenter);
    for (uint64_t i = 0; i < npix; ++i) keys[i] = ~(uint64_t)0;
    for (uint64_t ti = 0; ti < ntri; ++ti) {
        otri t;
        if (!tri_setup(clip + 12 * ti, width, height, &t)) continue;
        int xmin = t.x[0], xmax = t.x[0], ymin = t.y[0], ymax = t.y[0];
        for (int k = 1; k < 3; ++k) {
            xmin = t.x[k] < xmin ? t.x[k] : xmin;
            xmax = t.x[k] > xmax ? t.x[k] : xmax;
            ymin = t.y[k] < ymin ? t.y[k] : ymin;
            ymax = t.y[k] > ymax ? t.y[k] : ymax;
        }
        int x0 = floor_div256(xmin - 128 + 255), x1 = floor_div256(xmax - 128);
        int y0 = floor_div256(ymin - 128 + 255), y1 = floor_div256(ymax - 128);
        x0 = x0 < 0 ? 0 : x0;
        y0 = y0 < 0 ? 0 : y0;
        x1 = x1 > (int)width - 1 ? (int)width - 1 : x1;
        y1 = y1 > (int)height - 1 ? (int)height - 1 : y1;
        const int tl0 = top_left(t.x[1], t.y[1], t.x[2], t.y[2]), tl1 = top_left(t.x[2], t.y[2], t.x[0], t.y[0]),
                  tl2 = top_left(t.x[0], t.y[0], t.x[1], t.y[1]);
        for (int py = y0; py <= y1; ++py)
            for (int px = x0; px <= x1; ++px) {
                long long e[3];
                edges_at(&t, px, py, e);
                if (!((e[0] > 0 || (e[0] == 0 && tl0)) && (e[1] > 0 || (e[1] == 0 && tl1)) &&
                      (e[2] > 0 || (e[2] == 0 && tl2))))
                    continue;
                const float z = (((float)e[0] * t.z[0] + (float)e[1] * t.z[1]) + (float)e[2] * t.z[2]) / (float)t.area;
                if (!(z >= 0.0f && z < 1.0f)) continue;
                uint32_t zb;
                memcpy(&zb, &z, 4);
                const uint64_t key = ((uint64_t)zb << 32) | (uint32_t)ti;
                uint64_t* k = keys + (uint64_t)py * width + px;
                if (key < *k) *k = key;
            }
    }
    for (uint64_t i = 0; i < npix; ++i) {
        float out[4] = {1.0f, 1.0f, 1.0f, 1.0f}, dep = 1.0f;
        uint32_t tri = 0xffffffffu;
        if (keys[i] != ~(uint64_t)0) {
            const uint64_t t = keys[i] & 0xffffffffu;
            const uint32_t zb = (uint32_t)(keys[i] >> 32);
            tri = (uint32_t)t;
            memcpy(&dep, &zb, 4);
            otri tr;
            tri_setup(clip + 12 * t, width, height, &tr);
            long long ee[3];
            edges_at(&tr, (int)(i % width), (int)(i / width), ee);
            const float e[3] = {(float)ee[0], (float)ee[1], (float)ee[2]};
            float pw[3], psum = 0.0f;
            for (int k = 0; k < 3; ++k) {
                pw[k] = e[k] / clip[12 * t + 4 * tr.idx[k] + 3];
                psum = psum + pw[k];
            }
            float wp[3] = {0.0f, 0.0f, 0.0f};
            float te = 0.0f;
            for (int k = 0; k < 3; ++k) {
                const float b = pw[k] / psum;
                const float* wk = world + 3 * (3 * t + tr.idx[k]);
                for (int c = 0; c < 3; ++c) wp[c] = wp[c] + b * wk[c];
                if (fog) te = te + b * tenter[3 * t + tr.idx[k]];
            }
            bcmc_oracle_shade(wp, te, eye, world + 9 * t, fog, out);
        }
        for (int k = 0; k < 4; ++k) rgba[4 * i + k] = out[k];
        if (depth) depth[i] = dep;
        if (triangle) triangle[i] = tri;
    }
    free(world);
    free(clip);
    free(tenter);
    free(keys);
    return 0;
}

/* ======================================================================== */
/* compute_block_active.comp:24-61                                           */
/* ======================================================================== */
void bcmc_oracle_block_active(const float* ranges, const uint32_t dims[3], float iso,
                              uint32_t* active)
{
    const int32_t nbx = (int32_t)(align_to(dims[0], 4) / 4), nby = (int32_t)(align_to(dims[1], 4) / 4),
                  nbz = (int32_t)(align_to(dims[2], 4) / 4);
    const int64_t nblocks = (int64_t)nbx * nby * nbz;
#pragma omp parallel for schedule(static)
    for (int64_t bi = 0; bi < nblocks; ++bi) {
        const int32_t gx = (int32_t)(bi % nbx), gy = (int32_t)((bi / nbx) % nby),
                      gz = (int32_t)(bi / ((int64_t)nbx * nby));
        const float lo = ranges[2 * bi], hi = ranges[2 * bi + 1];
        uint32_t a = 0;
        if (iso >= lo && iso <= hi) {
            a = 1;
        } else {
            for (int k = -1; k < 2 && !a; ++k)
                for (int j = -1; j < 2 && !a; ++j)
                    for (int i = -1; i < 2 && !a; ++i) {
                        const int32_t cx = gx + i, cy = gy + j, cz = gz + k;
                        if ((i == 0 && j == 0 && k == 0) || cx < 0 || cy < 0 || cz < 0 || cx >= nbx ||
                            cy >= nby || cz >= nbz)
                            continue;
                        const int64_t n = cx + (int64_t)nbx * (cy + (int64_t)nby * cz);
                        const float ulo = glsl_min(lo, ranges[2 * n]);
                        const float uhi = glsl_max(hi, ranges[2 * n + 1]);
                        if (iso >= ulo && iso <= uhi) a = 1;
                    }
        }
        active[bi] = a;
    }
}

/* ======================================================================== */
/* exclusive_scan.js:178-295 / stream_compact.js:56-165                       */
/* ======================================================================== */
uint32_t bcmc_oracle_exclusive_scan(uint32_t* data, uint32_t n, uint32_t aligned_n)
{
    uint32_t sum = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t v = data[i];
        data[i] = sum;
        sum += v;
    }
    if (n < aligned_n) data[n] = sum;
    return sum;
}

void bcmc_oracle_compact(const uint32_t* flags, const uint32_t* offsets, uint32_t n, uint32_t* out)
{
    for (uint32_t i = 0; i < n; ++i)
        if (flags[i] != 0) out[offsets[i]] = i;
}

/* ======================================================================== */
/* RadixSorter (radix_sort_by_key.js:155-400): 64-element chunks sorted by  */
/* 32 one-bit stable splits (radix_sort_chunk.comp:28-101), log2 merge      */
/* passes with upper/lower bound placement (merge_sorted_chunks.comp:35-94), */
/* then an optional full reversal (reverse_buffer.comp:15-29) and readback  */
/* from alignedSize-size.  The reference's reversal races when the array is */
/* one chunk (n <= 64); the oracle performs the intended full reversal.     */
/* ======================================================================== */
#define SORT_CHUNK 64u

static uint32_t next_pow2_u32(uint32_t a)
{
    a = a - 1;
    a |= a >> 1; a |= a >> 2; a |= a >> 4; a |= a >> 8; a |= a >> 16;
    return a + 1;
}

uint32_t bcmc_oracle_sort_aligned_size(uint32_t n)
{
    return next_pow2_u32((n + SORT_CHUNK - 1) / SORT_CHUNK) * SORT_CHUNK;
}

static uint32_t upper_bound_u32(const uint32_t* k, uint32_t start, uint32_t count, uint32_t e)
{
    while (count > 0) {
        const uint32_t i = start + count / 2;
        if (e >= k[i]) { start = i + 1; count -= count / 2 + 1; }
        else count = count / 2;
    }
    return start;
}

static uint32_t lower_bound_u32(const uint32_t* k, uint32_t start, uint32_t count, uint32_t e)
{
    while (count > 0) {
        const uint32_t i = start + count / 2;
        if (k[i] < e) { start = i + 1; count -= count / 2 + 1; }
        else count = count / 2;
    }
    return start;
}

void bcmc_oracle_sort_by_key(uint32_t* keys, uint32_t* values, uint32_t size, int reverse)
{
    const uint32_t chunk_count = next_pow2_u32((size + SORT_CHUNK - 1) / SORT_CHUNK);
    const uint32_t aligned = chunk_count * SORT_CHUNK;
    uint32_t steps = 0;
    while ((1u << steps) < chunk_count) ++steps;
    uint32_t* sk = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    uint32_t* sv = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    /* chunk sort with UINT_MAX padding */
    for (uint32_t c = 0; c < chunk_count; ++c) {
        uint32_t kb[SORT_CHUNK], vb[SORT_CHUNK], tk[SORT_CHUNK], tv[SORT_CHUNK];
        for (uint32_t t = 0; t < SORT_CHUNK; ++t) {
            const uint32_t idx = c * SORT_CHUNK + t;
            kb[t] = idx < size ? keys[idx] : 0xffffffffu;
            vb[t] = idx < size ? values[idx] : 0xffffffffu;
        }
        for (uint32_t bit = 0; bit < 32; ++bit) {
            const uint32_t mask = 1u << bit;
            uint32_t total_false = 0;
            for (uint32_t t = 0; t < SORT_CHUNK; ++t) total_false += (kb[t] & mask) ? 0 : 1;
            uint32_t f = 0;
            for (uint32_t t = 0; t < SORT_CHUNK; ++t) {
                const uint32_t dst = (kb[t] & mask) ? t - f + total_false : f;
                tk[dst] = kb[t];
                tv[dst] = vb[t];
                f += (kb[t] & mask) ? 0 : 1;
            }
            memcpy(kb, tk, sizeof(kb));
            memcpy(vb, tv, sizeof(vb));
        }
        memcpy(keys + c * SORT_CHUNK, kb, sizeof(kb));
        memcpy(values + c * SORT_CHUNK, vb, sizeof(vb));
    }
    /* merges, ping-ponging between (keys,values) and scratch */
    uint32_t *ik = keys, *iv = values, *ok = sk, *ov = sv;
    for (uint32_t s = 0; s < steps; ++s) {
        const uint32_t groups = chunk_count / (2u << s);
        const uint32_t out_size = aligned / groups, half = out_size / 2;
        for (uint32_t g = 0; g < groups; ++g) {
            const uint32_t offs = g * out_size;
            for (uint32_t i = 0; i < half; ++i) {
                const uint32_t a_in = offs + i, b_in = offs + half + i;
                const uint32_t a_loc = i + upper_bound_u32(ik, offs + half, half, ik[a_in]) - half;
                const uint32_t b_loc = i + lower_bound_u32(ik, offs, half, ik[b_in]);
                ok[a_loc] = ik[a_in]; ov[a_loc] = iv[a_in];
                ok[b_loc] = ik[b_in]; ov[b_loc] = iv[b_in];
            }
        }
        uint32_t* t;
        t = ik; ik = ok; ok = t;
        t = iv; iv = ov; ov = t;
    }
    /* ik/iv hold the ascending order */
    uint32_t* rk = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    uint32_t* rv = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    if (reverse) {
        /* full reversal, then read back from alignedSize - size */
        for (uint32_t i = 0; i < size; ++i) {
            rv[i] = iv[size - 1 - i];
            rk[i] = ik[size - 1 - i];
        }
        memcpy(values, rv, sizeof(uint32_t) * size);
        memcpy(keys, rk, sizeof(uint32_t) * size);
    } else {
        memcpy(rv, iv, sizeof(uint32_t) * aligned);
        memcpy(rk, ik, sizeof(uint32_t) * aligned);
        memcpy(values, rv, sizeof(uint32_t) * aligned);
        memcpy(keys, rk, sizeof(uint32_t) * aligned);
    }
    free(rk);
    free(rv);
    free(sk);
    free(sv);
}

/* ======================================================================== */
/* LRUCache (lru_cache.js:4-903)                                             */
/* ======================================================================== */
struct bcmc_oracle_lru {
    uint32_t total, aligned_total, cache_size, element_size;
    int32_t* item_slot;  /* cachedItemSlots [aligned_total] */
    uint32_t* age;       /* slotData.age */
    uint32_t* avail;     /* slotData.available */
    int32_t* item;       /* slotData.item_id */
    float* cache;        /* cache_size * element_size bytes */
    uint32_t* needs;     /* needsCaching [aligned_total] */
    uint32_t display_slots_available;
    uint32_t* last_sorted;
    uint32_t last_sorted_n;
};

bcmc_oracle_lru* bcmc_oracle_lru_create(uint32_t initial_size, uint32_t element_size,
                                        uint32_t total)
{
    bcmc_oracle_lru* c = (bcmc_oracle_lru*)calloc(1, sizeof(*c));
    c->total = total;
    c->aligned_total = align_to(total, 32);
    c->cache_size = align_to(initial_size, 32);
    c->element_size = element_size;
    c->item_slot = (int32_t*)malloc(sizeof(int32_t) * c->aligned_total);
    c->needs = (uint32_t*)calloc(c->aligned_total, sizeof(uint32_t));
    for (uint32_t i = 0; i < c->aligned_total; ++i) c->item_slot[i] = -1;
    c->age = (uint32_t*)malloc(sizeof(uint32_t) * c->cache_size);
    c->avail = (uint32_t*)malloc(sizeof(uint32_t) * c->cache_size);
    c->item = (int32_t*)malloc(sizeof(int32_t) * c->cache_size);
    for (uint32_t i = 0; i < c->cache_size; ++i) {
        c->age[i] = 2 + i; /* lru_cache.js:54-59 */
        c->avail[i] = 1;
        c->item[i] = -1;
    }
    c->cache = (float*)calloc((size_t)c->cache_size * element_size / 4 + 1, sizeof(float));
    return c;
}

void bcmc_oracle_lru_destroy(bcmc_oracle_lru* c)
{
    if (!c) return;
    free(c->item_slot); free(c->needs); free(c->age); free(c->avail); free(c->item);
    free(c->cache); free(c->last_sorted); free(c);
}

uint32_t bcmc_oracle_lru_update(bcmc_oracle_lru* c, const uint32_t* item_needed,
                                uint32_t* new_item_ids)
{
    /* lru_cache_age_slots.comp:14-21 */
    for (uint32_t s = 0; s < c->cache_size; ++s) c->age[s] += 1;
    /* lru_cache_mark_new_items.comp:26-44 (items past `total` read as 0) */
    for (uint32_t i = 0; i < c->aligned_total; ++i) {
        const uint32_t needed = i < c->total ? item_needed[i] : 0;
        const int32_t slot = c->item_slot[i];
        if (slot >= 0) {
            c->needs[i] = 0;
            if (needed == 1) {
                c->age[slot] = 0;
                c->avail[slot] = 0;
            } else {
                c->avail[slot] = 1;
            }
        } else {
            c->needs[i] = needed;
        }
    }
    /* lru_cache.js:463-492: scan + compact the items that need caching */
    uint32_t num_new = 0;
    for (uint32_t i = 0; i < c->total; ++i)
        if (c->needs[i] != 0) new_item_ids[num_new++] = i;
    if (num_new == 0) return 0;
    /* lru_cache.js:501 */
    uint32_t num_avail = 0;
    for (uint32_t s = 0; s < c->cache_size; ++s) num_avail += c->avail[s];
    /* lru_cache.js:510-672: grow, lru_cache_init.comp:19-30 */
    if (num_avail < num_new) {
        uint64_t grown = (uint64_t)c->cache_size + (uint64_t)ceil((double)(num_new - num_avail) * 1.5);
        if (grown > c->total) grown = c->total;
        const uint32_t new_size = align_to((uint32_t)grown, 32);
        c->age = (uint32_t*)realloc(c->age, sizeof(uint32_t) * new_size);
        c->avail = (uint32_t*)realloc(c->avail, sizeof(uint32_t) * new_size);
        c->item = (int32_t*)realloc(c->item, sizeof(int32_t) * new_size);
        const size_t old_floats = (size_t)c->cache_size * c->element_size / 4;
        const size_t new_floats = (size_t)new_size * c->element_size / 4;
        c->cache = (float*)realloc(c->cache, sizeof(float) * (new_floats + 1));
        memset(c->cache + old_floats, 0, sizeof(float) * (new_floats + 1 - old_floats));
        for (uint32_t s = c->cache_size; s < new_size; ++s) {
            c->age[s] = 100000;
            c->avail[s] = 1;
            c->item[s] = -1;
        }
        c->cache_size = new_size;
        num_avail = 0;
        for (uint32_t s = 0; s < c->cache_size; ++s) num_avail += c->avail[s];
    }
    c->display_slots_available = num_avail - num_new;
    /* lru_cache.js:684-766: compact available slot ids, gather their ages */
    const uint32_t aligned = bcmc_oracle_sort_aligned_size(num_avail);
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * aligned);
    uint32_t p = 0;
    for (uint32_t s = 0; s < c->cache_size; ++s)
        if (c->avail[s]) ids[p++] = s;
    for (uint32_t i = 0; i < num_avail; ++i) keys[i] = c->age[ids[i]];
    /* lru_cache.js:769: oldest first */
    bcmc_oracle_sort_by_key(keys, ids, num_avail, 1);
    free(c->last_sorted);
    c->last_sorted = ids;
    c->last_sorted_n = num_avail;
    free(keys);
    /* lru_cache_update.comp:19-37 */
    for (uint32_t i = 0; i < num_new; ++i) {
        const uint32_t it = new_item_ids[i];
        const uint32_t slot = ids[i];
        const int32_t prev = c->item[slot];
        if (prev != -1) c->item_slot[prev] = -1;
        c->age[slot] = 0;
        c->item[slot] = (int32_t)it;
        c->avail[slot] = 0;
        c->item_slot[it] = (int32_t)slot;
    }
    return num_new;
}

/* lru_cache.js:846-903 */
void bcmc_oracle_lru_reset(bcmc_oracle_lru* c)
{
    for (uint32_t s = 0; s < c->cache_size; ++s) {
        c->age[s] = 100000;
        c->avail[s] = 1;
        c->item[s] = -1;
    }
    for (uint32_t i = 0; i < c->total; ++i) c->item_slot[i] = -1;
}

uint32_t bcmc_oracle_lru_cache_size(const bcmc_oracle_lru* c) { return c->cache_size; }
uint32_t bcmc_oracle_lru_slots_available(const bcmc_oracle_lru* c) { return c->display_slots_available; }
const int32_t* bcmc_oracle_lru_item_slots(const bcmc_oracle_lru* c) { return c->item_slot; }
const uint32_t* bcmc_oracle_lru_slot_age(const bcmc_oracle_lru* c) { return c->age; }
const uint32_t* bcmc_oracle_lru_slot_avail(const bcmc_oracle_lru* c) { return c->avail; }
const int32_t* bcmc_oracle_lru_slot_item(const bcmc_oracle_lru* c) { return c->item; }
float* bcmc_oracle_lru_cache_data(bcmc_oracle_lru* c) { return c->cache; }
const uint32_t* bcmc_oracle_lru_last_sorted(const bcmc_oracle_lru* c, uint32_t* n)
{
    *n = c->last_sorted_n;
    return c->last_sorted;
}

/* ======================================================================== */
/* Marching cubes over cached blocks (compute_vertex_values.comp,            */
/* compute_block_has_vertices.comp, compute_block_voxel_num_verts.comp,      */
/* compute_block_vertices.comp, block_vertex_position.comp)                  */
/* ======================================================================== */
static const uint32_t kIndexToVertex[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const uint32_t kEdgeVertices[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {6, 5},
                                              {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

typedef struct {
    uint32_t nb[3];
    const uint32_t* active;
    const int32_t* slots;
    const float* cache;
} mc_view;

static inline uint32_t block_id_of(const mc_view* v, uint32_t x, uint32_t y, uint32_t z)
{
    return x + v->nb[0] * (y + v->nb[1] * z);
}

/* compute_vertex_values.comp:96-156 */
static void block_dims_with_ghost(const mc_view* v, const uint32_t bp[3], uint32_t d[3])
{
    d[0] = d[1] = d[2] = 4;
    if (bp[0] + 1 < v->nb[0]) d[0] = 5;
    if (bp[1] + 1 < v->nb[1]) d[1] = 5;
    if (bp[2] + 1 < v->nb[2]) d[2] = 5;
    if (d[0] == 5 && d[1] == 5 && d[2] == 5) {
        if (v->active[block_id_of(v, bp[0] + 1, bp[1] + 1, bp[2] + 1)] == 0) d[0] = d[1] = d[2] = 4;
    }
    if (d[0] == 5 && d[1] == 5) {
        if (v->active[block_id_of(v, bp[0] + 1, bp[1] + 1, bp[2])] == 0) d[0] = d[1] = 4;
    }
    if (d[0] == 5 && d[2] == 5) {
        if (v->active[block_id_of(v, bp[0] + 1, bp[1], bp[2] + 1)] == 0) d[0] = d[2] = 4;
    }
    if (d[1] == 5 && d[2] == 5) {
        if (v->active[block_id_of(v, bp[0], bp[1] + 1, bp[2] + 1)] == 0) d[1] = d[2] = 4;
    }
    if (d[0] == 5 && v->active[block_id_of(v, bp[0] + 1, bp[1], bp[2])] == 0) d[0] = 4;
    if (d[1] == 5 && v->active[block_id_of(v, bp[0], bp[1] + 1, bp[2])] == 0) d[1] = 4;
    if (d[2] == 5 && v->active[block_id_of(v, bp[0], bp[1], bp[2] + 1)] == 0) d[2] = 4;
}

/* compute_vertex_values.comp:158-252: fill vol[128] for block `id` */
static void load_block(const mc_view* v, uint32_t id, float vol[128], uint32_t d[3], uint32_t bp[3])
{
    for (int i = 0; i < 128; ++i) vol[i] = 0.0f;
    bp[0] = id % v->nb[0];
    bp[1] = (id / v->nb[0]) % v->nb[1];
    bp[2] = id / (v->nb[0] * v->nb[1]);
    block_dims_with_ghost(v, bp, d);
    for (uint32_t z = 0; z < d[2]; ++z)
        for (uint32_t y = 0; y < d[1]; ++y)
            for (uint32_t x = 0; x < d[0]; ++x) {
                /* the voxel comes from whichever block holds it */
                const uint32_t ox = x / 4, oy = y / 4, oz = z / 4;
                const uint32_t nid = block_id_of(v, bp[0] + ox, bp[1] + oy, bp[2] + oz);
                const int32_t slot = v->slots[nid];
                const uint32_t lv = (x % 4) + 4 * ((y % 4) + 4 * (z % 4));
                vol[x + d[0] * (y + d[1] * z)] = v->cache[(uint64_t)(uint32_t)slot * 64u + lv];
            }
}

/* per-cell case index (compute_block_has_vertices.comp:28-40) */
static inline uint32_t cell_case(const float vol[128], const uint32_t d[3], uint32_t cell, float iso,
                                 float values[8])
{
    const uint32_t px = cell % 4, py = (cell / 4) % 4, pz = cell / 16;
    uint32_t ci = 0;
    for (int i = 0; i < 8; ++i) {
        const uint32_t* o = kIndexToVertex[i];
        const uint32_t vx = ((pz + o[2]) * d[1] + py + o[1]) * d[0] + px + o[0];
        values[i] = vol[vx];
        if (values[i] <= iso) ci |= 1u << i;
    }
    return ci;
}

static inline int cell_valid(const uint32_t d[3], uint32_t cell)
{
    return (cell % 4) + 1 < d[0] && ((cell / 4) % 4) + 1 < d[1] && (cell / 16) + 1 < d[2];
}

static uint32_t block_vertex_count(const mc_view* v, uint32_t id, float iso)
{
    float vol[128], values[8];
    uint32_t d[3], bp[3], n = 0;
    load_block(v, id, vol, d, bp);
    for (uint32_t cell = 0; cell < 64; ++cell)
        if (cell_valid(d, cell)) n += g_case_count[cell_case(vol, d, cell, iso, values)];
    return n;
}

/* block_vertex_position.comp:9-17 */
static inline uint32_t compress_position(const float p[3])
{
    uint32_t q[3];
    for (int i = 0; i < 3; ++i) {
        /* WGSL u32(f32): truncate toward zero, saturating (NaN -> 0) */
        const float f = ((p[i] - 0.5f) * 0.25f) * 1023.0f;
        q[i] = !(f > 0.0f) ? 0u : (f >= 4294967296.0f ? 0xffffffffu : (uint32_t)f);
    }
    return ((q[0] & 0x3ffu) << 20) | ((q[1] & 0x3ffu) << 10) | (q[2] & 0x3ffu);
}

/* compute_block_vertices.comp:62-174 */
static void block_emit(const mc_view* v, uint32_t id, float iso, uint32_t offset, uint32_t* verts)
{
    float vol[128], values[8];
    uint32_t d[3], bp[3];
    load_block(v, id, vol, d, bp);
    uint32_t local = 0;
    for (uint32_t cell = 0; cell < 64; ++cell) {
        if (!cell_valid(d, cell)) continue;
        const uint32_t ci = cell_case(vol, d, cell, iso, values);
        const float vp[3] = {(float)(cell % 4), (float)((cell / 4) % 4), (float)(cell / 16)};
        const int32_t* row = g_tri[ci];
        uint32_t t;
        for (t = 0; row[t] != -1; ++t) {
            const uint32_t v0 = kEdgeVertices[row[t]][0], v1 = kEdgeVertices[row[t]][1];
            const float fa = values[v0], fb = values[v1];
            float tt;
            if (fabsf(fa - fb) < 0.001f) tt = 0.0f;
            else tt = (iso - fa) / (fb - fa);
            float p[3];
            for (int k = 0; k < 3; ++k) {
                const int32_t a = (int32_t)kIndexToVertex[v0][k], b = (int32_t)kIndexToVertex[v1][k];
                const float lerp = (float)a + tt * (float)(b - a);
                p[k] = (lerp + vp[k]) + 0.5f;
            }
            const uint64_t o = (uint64_t)offset + local + t;
            verts[2 * o] = compress_position(p);
            verts[2 * o + 1] = id;
        }
        local += t;
    }
}

/* ======================================================================== */
/* CompressedMarchingCubes (compressed_marching_cubes.js:1-1122)             */
/* ======================================================================== */
struct bcmc_oracle_mc {
    const uint64_t* words;
    uint32_t dims[3], padded[3], nb[3], total_blocks, max_bits;
    float scale[3];
    float* ranges;
    uint32_t* active;
    uint32_t* active_offsets;
    uint32_t* active_ids;
    uint32_t* has_verts;
    uint32_t* with_verts;
    uint32_t* vert_offsets;
    uint32_t* new_items;
    uint32_t* verts;
    uint64_t verts_cap;
    bcmc_oracle_lru* lru;
    /* the reference object's fields, updated where it updates them */
    uint32_t num_active, num_with_verts, num_verts, new_decompressed;
};

bcmc_oracle_mc* bcmc_oracle_mc_create(const uint64_t* words, uint64_t nwords, uint32_t rate,
                                      const uint32_t dims[3], const float scale[3],
                                      double initial_cache_fraction)
{
    (void)nwords;
    init_tables();
    bcmc_oracle_mc* m = (bcmc_oracle_mc*)calloc(1, sizeof(*m));
    m->words = words;
    for (int i = 0; i < 3; ++i) {
        m->dims[i] = dims[i];
        m->padded[i] = align_to(dims[i], 4);
        m->nb[i] = m->padded[i] / 4;
        m->scale[i] = scale ? scale[i] : 1.0f;
    }
    m->total_blocks = m->nb[0] * m->nb[1] * m->nb[2];
    m->max_bits = 64u * rate;
    /* compressed_marching_cubes.js:443-448: initial cache = ceil(5% of blocks) */
    const uint32_t init = (uint32_t)ceil((double)m->total_blocks * initial_cache_fraction);
    m->lru = bcmc_oracle_lru_create(init, 256, m->total_blocks);
    const uint32_t n = m->total_blocks;
    m->ranges = (float*)malloc(sizeof(float) * 2 * n);
    m->active = (uint32_t*)calloc(n, sizeof(uint32_t));
    m->active_offsets = (uint32_t*)calloc(align_to(n, 512) + 1, sizeof(uint32_t));
    m->active_ids = (uint32_t*)calloc(n, sizeof(uint32_t));
    m->has_verts = (uint32_t*)calloc(align_to(n, 512) + 1, sizeof(uint32_t));
    m->with_verts = (uint32_t*)calloc(n, sizeof(uint32_t));
    m->vert_offsets = (uint32_t*)calloc(align_to(n, 512) + 1, sizeof(uint32_t));
    m->new_items = (uint32_t*)calloc(n, sizeof(uint32_t));
    bcmc_oracle_block_ranges(words, dims, m->max_bits, m->ranges);
    return m;
}

void bcmc_oracle_mc_destroy(bcmc_oracle_mc* m)
{
    if (!m) return;
    bcmc_oracle_lru_destroy(m->lru);
    free(m->ranges); free(m->active); free(m->active_offsets); free(m->active_ids);
    free(m->has_verts); free(m->with_verts); free(m->vert_offsets); free(m->new_items);
    free(m->verts); free(m);
}

uint32_t bcmc_oracle_mc_compute_surface(bcmc_oracle_mc* m, float iso)
{
    const uint32_t n = m->total_blocks;
    /* computeActiveBlocks (:811-829) */
    bcmc_oracle_block_active(m->ranges, m->dims, iso, m->active);
    memcpy(m->active_offsets, m->active, sizeof(uint32_t) * n);
    const uint32_t num_active = bcmc_oracle_exclusive_scan(m->active_offsets, n, align_to(n, 512));
    if (num_active == 0) return 0; /* :630-641, no cache update */
    /* lruCache.update (:648-649) and decompressBlocks (:689-694) */
    const uint32_t num_new = bcmc_oracle_lru_update(m->lru, m->active, m->new_items);
    m->new_decompressed = num_new;
    m->num_active = num_active;
    {
        float* cache = bcmc_oracle_lru_cache_data(m->lru);
        const int32_t* slots = bcmc_oracle_lru_item_slots(m->lru);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)num_new; ++i) {
            const uint32_t b = m->new_items[i];
            bcmc_oracle_decode_block(m->words, b, m->max_bits, 0,
                                     cache + (uint64_t)(uint32_t)slots[b] * 64u);
        }
    }
    /* compactActiveIDs (:704-707) */
    bcmc_oracle_compact(m->active, m->active_offsets, n, m->active_ids);
    mc_view v = {{m->nb[0], m->nb[1], m->nb[2]}, m->active, bcmc_oracle_lru_item_slots(m->lru),
                 bcmc_oracle_lru_cache_data(m->lru)};
    /* computeBlockHasVertices (:915-991) */
    uint32_t* counts = (uint32_t*)malloc(sizeof(uint32_t) * (num_active + 1));
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)num_active; ++i) {
        counts[i] = block_vertex_count(&v, m->active_ids[i], iso);
        m->has_verts[i] = counts[i] > 0 ? 1u : 0u;
    }
    /* scan + compact blocks with vertices (:721-756) */
    uint32_t* hv_offsets = (uint32_t*)malloc(sizeof(uint32_t) * (align_to(num_active, 512) + 1));
    memcpy(hv_offsets, m->has_verts, sizeof(uint32_t) * num_active);
    const uint32_t num_wv = bcmc_oracle_exclusive_scan(hv_offsets, num_active, align_to(num_active, 512));
    m->num_with_verts = num_wv;
    bcmc_oracle_compact(m->has_verts, hv_offsets, num_active, m->with_verts);
    free(hv_offsets);
    /* computeBlockVertexCounts (:993-1042) */
    for (uint32_t i = 0; i < num_wv; ++i) m->vert_offsets[i] = counts[m->with_verts[i]];
    const uint32_t num_verts = bcmc_oracle_exclusive_scan(m->vert_offsets, num_wv, align_to(num_wv, 512));
    free(counts);
    if (num_verts == 0) return 0; /* :769-772 */
    m->num_verts = num_verts;
    if (num_verts > m->verts_cap) {
        free(m->verts);
        m->verts_cap = num_verts;
        m->verts = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)num_verts);
    }
    /* computeVertices (:1044-1122) */
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)num_wv; ++i)
        block_emit(&v, m->active_ids[m->with_verts[i]], iso, m->vert_offsets[i], m->verts);
    return num_verts;
}

void bcmc_oracle_mc_cache_reset(bcmc_oracle_mc* m) { bcmc_oracle_lru_reset(m->lru); }
bcmc_oracle_lru* bcmc_oracle_mc_lru(bcmc_oracle_mc* m) { return m->lru; }
const uint32_t* bcmc_oracle_mc_vertices(const bcmc_oracle_mc* m) { return m->verts; }
const float* bcmc_oracle_mc_ranges(const bcmc_oracle_mc* m) { return m->ranges; }
const uint32_t* bcmc_oracle_mc_active(const bcmc_oracle_mc* m) { return m->active; }
const uint32_t* bcmc_oracle_mc_active_ids(const bcmc_oracle_mc* m) { return m->active_ids; }
const uint32_t* bcmc_oracle_mc_with_verts(const bcmc_oracle_mc* m) { return m->with_verts; }
const uint32_t* bcmc_oracle_mc_vert_offsets(const bcmc_oracle_mc* m) { return m->vert_offsets; }
const uint32_t* bcmc_oracle_mc_new_items(const bcmc_oracle_mc* m) { return m->new_items; }

void bcmc_oracle_mc_stats(const bcmc_oracle_mc* m, uint32_t stats[7])
{
    stats[0] = m->total_blocks;
    stats[1] = m->num_active;
    stats[2] = m->new_decompressed;
    stats[3] = m->num_with_verts;
    stats[4] = m->num_verts;
    stats[5] = bcmc_oracle_lru_cache_size(m->lru);
    stats[6] = bcmc_oracle_lru_slots_available(m->lru);
}
