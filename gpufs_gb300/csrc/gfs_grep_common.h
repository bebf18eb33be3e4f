/*
 * Token hashing shared by the host-side dictionary builder and the device
 * scanner of grep_text, so both place a word in the same buckets.
 *
 * A token is a maximal run of [A-Za-z_] (samples/grep_text/grep_text_gpu.cu:79);
 * its key is the token bytes zero-padded to 32 bytes, i.e. exactly a
 * normalised 32-byte dictionary record (grep_text_gpu.cu:221: records are
 * 32 bytes, NUL padded), as 8 little-endian 32-bit words.
 *
 * The hash is 32-bit integer arithmetic only (a multiply-add over the key
 * words, one xor-shift-multiply round, and one more multiply for the second
 * bucket): a handful of instructions per token on the GPU, where the scan is
 * instruction-bound.
 */
#ifndef GFS_GREP_COMMON_H
#define GFS_GREP_COMMON_H

#include <stdint.h>

#ifdef __CUDACC__
#define GFS_HD __host__ __device__ __forceinline__
#else
#define GFS_HD static inline
#endif

#define GREP_WAYS 4         /* slots per bucket */
#define GREP_TAG_LONG 0x8000u /* tag bit: the word has 17..32 letters */

/* key words k[0..7], len in 1..32 */
GFS_HD uint32_t grep_mix(const uint32_t k[8], int len) {
    uint32_t a = (uint32_t)len * 0x9E3779B1u + k[0] * 0x85EBCA77u + k[1] * 0xC2B2AE3Du + k[2] * 0x27D4EB2Fu +
                 k[3] * 0x165667B1u;
    if (len > 16) a += k[4] * 0xD3A2646Du + k[5] * 0xFD7046C5u + k[6] * 0xB55A4F09u + k[7] * 0x8DA6B343u;
    return a;
}
GFS_HD uint32_t grep_h1(uint32_t a) { return (a ^ (a >> 15)) * 0x2C1B3C6Du; }
/* 16-bit slot tag, never 0 (0 marks an empty slot): 15 hash bits, and the
 * top bit set for words of 17..32 letters, so a token of at most 16 letters
 * never meets a longer word's slot */
GFS_HD uint32_t grep_tag(uint32_t h1, int len) {
    uint32_t t = (h1 & 0x7FFFu) | (len > 16 ? GREP_TAG_LONG : 0u);
    return t ? t : 1u;
}
GFS_HD uint32_t grep_bucket(uint32_t h, uint32_t nb) { return (uint32_t)(((uint64_t)h * nb) >> 32); }
/* second bucket: the top bits of another multiple of h1 (it may equal the
 * first; the table builder then has only one bucket for the word) */
GFS_HD uint32_t grep_b2(uint32_t h1, uint32_t nb) { return grep_bucket(h1 * 0x85EBCA6Bu, nb); }

#endif
