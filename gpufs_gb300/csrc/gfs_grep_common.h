/*
 * Token hashing and the dictionary table layout, shared by the host-side
 * table builder, the device builder and the device scanners of grep_text, so
 * all of them place a word in the same slot.
 *
 * A token is a maximal run of [A-Za-z_] (samples/grep_text/grep_text_gpu.cu:79);
 * its key is the token bytes zero-padded to 32 bytes, i.e. exactly a
 * normalised 32-byte dictionary record (grep_text_gpu.cu:221: records are
 * 32 bytes, NUL padded), as 8 little-endian 32-bit words.
 *
 * The table is a hash-and-displace perfect hash over the dictionary's
 * distinct words (the published CHD scheme of Belazzougui, Botelho and
 * Dietzfelbinger, "Hash, displace, and compress", 2009, in a simplified
 * form): a word's 32-bit hash h picks one of r buckets; every bucket holds a
 * 16-bit displacement d, chosen at build time so that the words of all
 * buckets land in distinct slots of an m-slot array:
 *
 *     bucket = hi32(h * r)      slot = hi32(((h ^ d[bucket]) * GREP_SLOT_MUL) * m)
 *
 * A scan looks a token up with one displacement load, one 16-bit tag load
 * and one compare; a tag hit is verified against the slot's record.  Two
 * distinct words with the same h cannot be separated by any displacement, so
 * the mixing multipliers are seeded and the build moves to the next seed
 * when that happens (about one dictionary of 20,000 words in twenty).
 *
 * All arithmetic is 32-bit integer: a multiply-add over the key words with
 * the seeded multipliers, one xor-shift-multiply round, and the slot mix.
 */
#ifndef GFS_GREP_COMMON_H
#define GFS_GREP_COMMON_H

#include <stdint.h>

#ifdef __CUDACC__
#define GFS_HD __host__ __device__ __forceinline__
#else
#define GFS_HD static inline
#endif

#define GREP_TAG_LONG 0x8000u     /* tag bit: the word has 17..32 letters */
#define GREP_SLOT_MUL 0x9E3779B1u /* slot mix after the displacement */
#define GREP_BUCKET_LOAD 4        /* words per displacement bucket, on average */
#define GREP_SLOT_LOAD 0.88       /* words per slot */
#define GREP_MAX_BUCKET 32        /* a larger bucket fails the seed */

/* Seeded multipliers of the key mix: c[0] for the length, c[1..8] for the
 * key words.  All odd. */
struct grep_hashk {
    uint32_t c[9];
};

GFS_HD void grep_hash_seed(uint32_t seed, struct grep_hashk* hk) {
    /* a splitmix-style sequence from the seed */
    uint32_t x = seed * 0x9E3779B9u + 0x7F4A7C15u;
    for (int i = 0; i < 9; i++) {
        x += 0x9E3779B9u;
        uint32_t z = x;
        z = (z ^ (z >> 16)) * 0x85EBCA6Bu;
        z = (z ^ (z >> 13)) * 0xC2B2AE35u;
        z ^= z >> 16;
        hk->c[i] = z | 1u;
    }
}

/* key words k[0..7], len in 1..32 (for len <= 16, k[4..7] are zero and the
 * second half of the sum vanishes, so the device drops it) */
GFS_HD uint32_t grep_mix(const struct grep_hashk* hk, const uint32_t k[8], int len) {
    uint32_t a = (uint32_t)len * hk->c[0] + k[0] * hk->c[1] + k[1] * hk->c[2] + k[2] * hk->c[3] + k[3] * hk->c[4];
    if (len > 16) a += k[4] * hk->c[5] + k[5] * hk->c[6] + k[6] * hk->c[7] + k[7] * hk->c[8];
    return a;
}
GFS_HD uint32_t grep_h1(uint32_t a) { return (a ^ (a >> 15)) * 0x2C1B3C6Du; }
/* 16-bit slot tag, never 0 (0 marks an empty slot): 14 hash bits, bit 0 set,
 * and the top bit set for words of 17..32 letters, so a token of at most 16
 * letters never meets a longer word's slot */
GFS_HD uint32_t grep_tag(uint32_t h, int len) { return ((h | 1u) & 0x7FFFu) | (len > 16 ? GREP_TAG_LONG : 0u); }
GFS_HD uint32_t grep_hi(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }
GFS_HD uint32_t grep_bucket(uint32_t h, uint32_t r) { return grep_hi(h, r); }
GFS_HD uint32_t grep_slot(uint32_t h, uint32_t d, uint32_t m) { return grep_hi((h ^ d) * GREP_SLOT_MUL, m); }

/* Table geometry for n dictionary records: m slots, r displacement buckets. */
GFS_HD void grep_geometry(uint32_t n, uint32_t* m, uint32_t* r) {
    *m = (uint32_t)((double)n / GREP_SLOT_LOAD) + 16u;
    *r = n / GREP_BUCKET_LOAD + 1u;
}

#endif
