/*
 * XXH64 device primitives, written from the public xxHash specification
 * (XXH64: four 64-bit accumulators over 32-byte stripes, then a merge, the
 * length, the tail of < 32 bytes and an avalanche).  Used by the per-file
 * checksum kernel and by the batched scan, which hash bytes as they stream
 * through shared memory.
 */
#ifndef GFS_XXH64_CUH
#define GFS_XXH64_CUH

#include <stdint.h>

namespace gfsx {
namespace { /* internal linkage: every TU gets its own copy */

constexpr uint64_t P1 = 0x9E3779B185EBCA87ULL;
constexpr uint64_t P2 = 0xC2B2AE3D27D4EB4FULL;
constexpr uint64_t P3 = 0x165667B19E3779F9ULL;
constexpr uint64_t P4 = 0x85EBCA77C2B2AE63ULL;
constexpr uint64_t P5 = 0x27D4EB2F165667C5ULL;

__device__ __forceinline__ uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
__device__ __forceinline__ uint64_t round1(uint64_t acc, uint64_t in) {
    acc += in * P2;
    acc = rotl(acc, 31);
    return acc * P1;
}
__device__ __forceinline__ uint64_t merge(uint64_t acc, uint64_t v) {
    acc ^= round1(0, v);
    return acc * P1 + P4;
}
/* accumulator `lane` (0..3) at the start of a stream, seed 0 */
__device__ __forceinline__ uint64_t acc_init(int lane) {
    return lane == 0 ? P1 + P2 : lane == 1 ? P2 : lane == 2 ? 0ULL : 0ULL - P1;
}
/* `stripes` 32-byte stripes at p (8-byte aligned) into accumulator `lane` */
__device__ __forceinline__ uint64_t acc_stripes(uint64_t v, const uint8_t* p, uint32_t stripes, int lane) {
    const uint64_t* q = (const uint64_t*)p + lane;
    uint32_t s = 0;
    for (; s + 2 <= stripes; s += 2) {
        const uint64_t a = q[4 * s], b = q[4 * s + 4];
        v = round1(v, a);
        v = round1(v, b);
    }
    if (s < stripes) v = round1(v, q[4 * s]);
    return v;
}
/* the final hash of a stream of `len` bytes: accumulators v1..v4 (unused
 * when len < 32) and the last len % 32 bytes at tail (byte reads) */
__device__ __forceinline__ uint64_t finish(uint64_t v1, uint64_t v2, uint64_t v3, uint64_t v4, uint64_t len,
                                           const uint8_t* tail) {
    uint64_t h;
    if (len >= 32) {
        h = rotl(v1, 1) + rotl(v2, 7) + rotl(v3, 12) + rotl(v4, 18);
        h = merge(h, v1);
        h = merge(h, v2);
        h = merge(h, v3);
        h = merge(h, v4);
    } else {
        h = P5;
    }
    h += len;
    const uint32_t tn = (uint32_t)(len & 31u);
    uint32_t i = 0;
    for (; i + 8 <= tn; i += 8) {
        uint64_t k = 0;
        for (int b = 7; b >= 0; b--) k = (k << 8) | tail[i + b];
        h ^= round1(0, k);
        h = rotl(h, 27) * P1 + P4;
    }
    if (i + 4 <= tn) {
        const uint64_t k = (uint64_t)tail[i] | ((uint64_t)tail[i + 1] << 8) | ((uint64_t)tail[i + 2] << 16) |
                           ((uint64_t)tail[i + 3] << 24);
        h ^= k * P1;
        h = rotl(h, 23) * P2 + P3;
        i += 4;
    }
    for (; i < tn; i++) {
        h ^= (uint64_t)tail[i] * P5;
        h = rotl(h, 11) * P1;
    }
    h ^= h >> 33;
    h *= P2;
    h ^= h >> 29;
    h *= P3;
    h ^= h >> 32;
    return h;
}

} // namespace
} // namespace gfsx

#endif
