/*
 * Token hashing shared by the host-side dictionary builder and the device
 * scanner of grep_text, so both place a word in the same buckets.
 *
 * A token is a maximal run of [A-Za-z_] (samples/grep_text/grep_text_gpu.cu:79);
 * its key is the token bytes zero-padded to 32 bytes, i.e. exactly a
 * normalised 32-byte dictionary record (grep_text_gpu.cu:221: records are
 * 32 bytes, NUL padded), as 8 little-endian 32-bit words.
 */
#ifndef GFS_GREP_COMMON_H
#define GFS_GREP_COMMON_H

#include <stdint.h>

#ifdef __CUDACC__
#define GFS_HD __host__ __device__ __forceinline__
#else
#define GFS_HD static inline
#endif

#define GREP_WAYS 4       /* slots per bucket (16 bytes) */
#define GREP_TAG_SHIFT 20 /* slot word: tag:12 << 20 | count:20 */
#define GREP_CNT_MASK 0xFFFFFu

GFS_HD uint64_t grep_hash(const uint32_t k[8], int len) {
    const uint64_t K0 = 0x9E3779B97F4A7C15ULL, K1 = 0xD6E8FEB86659FD93ULL, K2 = 0xFF51AFD7ED558CCDULL;
    uint64_t h = (uint64_t)len * K0;
    h = (h ^ ((uint64_t)k[0] | ((uint64_t)k[1] << 32))) * K1;
    h ^= h >> 29;
    if (len > 8) {
        h = (h ^ ((uint64_t)k[2] | ((uint64_t)k[3] << 32))) * K1;
        h ^= h >> 29;
    }
    if (len > 16) {
        h = (h ^ ((uint64_t)k[4] | ((uint64_t)k[5] << 32))) * K1;
        h ^= h >> 29;
    }
    if (len > 24) {
        h = (h ^ ((uint64_t)k[6] | ((uint64_t)k[7] << 32))) * K1;
        h ^= h >> 29;
    }
    h ^= h >> 32;
    h *= K2;
    h ^= h >> 29;
    return h;
}

GFS_HD uint32_t grep_tag(uint64_t h) {
    uint32_t t = (uint32_t)(h >> 20) & 0xFFFu;
    return t ? t : 1u;
}
GFS_HD uint32_t grep_b1(uint64_t h, uint32_t nb) { return (uint32_t)(((uint64_t)(uint32_t)h * nb) >> 32); }
GFS_HD uint32_t grep_b2(uint64_t h, uint32_t nb) {
    uint32_t b = (uint32_t)(((h >> 32) * (uint64_t)nb) >> 32);
    uint32_t a = grep_b1(h, nb);
    return b == a ? (a + 1u == nb ? 0u : a + 1u) : b;
}

#endif
