// The device ZFP decoder (zfp_decode_staged: parse, deposit, transform) and
// encoder (zfp_encode_block with its bit writer) built as host code, one
// block at a time, for the CPU tests against the oracle.
#include "cuda_host_shim.h"
#include "zfp_device.cuh"

extern "C" void decode_blocks_host(const uint64_t* words, uint64_t nblocks, uint32_t rate, float* out)
{
    // the decoder reads 32-bit words and up to two words past a block
    const uint64_t n32 = nblocks * 2u * rate;
    uint32_t* w = new uint32_t[n32 + 8];
    memcpy(w, words, n32 * 4u);
    memset(w + n32, 0, 8 * 4);
    alignas(16) uint32_t pl[64];
    for (uint64_t b = 0; b < nblocks; ++b) bcmc::zfp_decode_staged(w + b * 2u * rate, 64u * rate, pl, out + b * 64u);
    delete[] w;
}

// `blocks`: nblocks gathered 4^3 blocks of 64 floats (x fastest, then y, z),
// as k_encode gathers them; `words` (nblocks * rate, zeroed) receives the
// fixed-rate stream.
extern "C" void encode_blocks_host(const float* blocks, uint64_t nblocks, uint32_t rate, unsigned long long* words)
{
    const uint32_t max_bits = 64u * rate;
    for (uint64_t b = 0; b < nblocks; ++b) {
        bcmc::BitWriter bw;
        bw.init(words, b * max_bits);
        bcmc::zfp_encode_block(blocks + b * 64u, max_bits, bw);
        bw.finish();
    }
}
