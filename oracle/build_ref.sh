#!/bin/sh
# Builds oracle/_ref/ from the reference sources where they lie (read-only).
# Test infrastructure only: the products are checkers, never shipped code.
#
#   libref_grep.so  the reference's own device matcher, `alpha` and
#                   `match_string` (samples/grep_text/grep_text_gpu.cu:79 and
#                   :139-160), cut out of the .cu by line range and compiled
#                   for the host with __device__ defined away.  The generated
#                   C file is kept beside it so a machine without the
#                   reference tree can recompile it (it stays git-ignored).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#        oracle/build_ref.sh --print-root    (prints where the tree is looked for)
# The root is the argument, else $GPUFS_REFERENCE, else /root/reference (the
# read-only copy of the reference tree on the build machine; it is absent
# where the tests run on a GPU, which need none of it).
set -eu
if [ "${1:-}" = "--print-root" ]; then
  echo "${GPUFS_REFERENCE:-/root/reference}"
  exit 0
fi
REF=${1:-${GPUFS_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/samples/grep_text/grep_text_gpu.cu"
[ -f "$SRC" ] || { echo "reference not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
GEN="$OUT/ref_match_string.c"
{
  echo "/* generated by oracle/build_ref.sh from samples/grep_text/grep_text_gpu.cu */"
  echo "#define __device__"
  sed -n '79p' "$SRC"
  sed -n '139,160p' "$SRC"
  cat <<'C'
/* a33: 33-byte word buffer (record + NUL), as orc_grep_match_string takes */
int ref_match_string(const char* a33, const char* data, int n) {
    char wl = 0;
    return match_string((char*)a33, (char*)data, n, &wl);
}

/* The reference's CPU-side work for grep_text, timed as its CPU path: every
 * dictionary record rescans every file through the window walk of
 * grep_text_gpu.cu:298-329 (16384+32-byte windows, overlap stitching, NUL
 * after the last window) calling the reference match_string above; records
 * are spread over nthreads host threads. */
#include <pthread.h>
#include <string.h>
#include <stdlib.h>
typedef struct { const unsigned char* dict; int n_words; const unsigned char* const* files;
                 const unsigned long long* sizes; int n_files; unsigned int* counts; int tid, nt; } rg_job;
static int rg_alpha(unsigned char c) { return (c >= 65 && c <= 90) || (c >= 97 && c <= 122) || c == 95; }
static void* rg_worker(void* p) {
    rg_job* j = (rg_job*)p;
    char* corpus = (char*)malloc(16384 + 32 + 1);
    for (int w = j->tid; w < j->n_words; w += j->nt) {
        char a[33];
        memcpy(a, j->dict + (size_t)w * 32, 32);
        a[32] = 0;
        for (int f = 0; f < j->n_files; f++) {
            unsigned long long size = j->sizes[f], cursor = 0, total = 0;
            while (cursor < size) {
                int last = size - cursor < 16384 + 32;
                int left = last ? (int)(size - cursor) : 16384 + 32;
                memcpy(corpus, j->files[f] + cursor, (size_t)left);
                corpus[left] = 0;
                int ov = 0;
                if (!last) { while (ov < 32 && rg_alpha((unsigned char)corpus[16384 + ov])) ov++; cursor += ov; }
                cursor += 16384;
                char wl;
                int m = match_string(a, corpus, last ? left + 1 : 16384 + ov + 1, &wl);
                if (m > 0) total += (unsigned long long)m;
            }
            j->counts[(size_t)w * j->n_files + f] = (unsigned int)total;
        }
    }
    free(corpus);
    return 0;
}
int ref_grep_counts(const unsigned char* dict, int n_words, const unsigned char* const* files,
                    const unsigned long long* sizes, int n_files, unsigned int* counts, int nthreads) {
    pthread_t th[256];
    rg_job jobs[256];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) {
        rg_job x = {dict, n_words, files, sizes, n_files, counts, t, nthreads};
        jobs[t] = x;
        pthread_create(&th[t], 0, rg_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], 0);
    return 0;
}
C
} > "$GEN"
${CC:-gcc} -O2 -shared -fPIC -pthread -o "$OUT/libref_grep.so" "$GEN"
echo "built $OUT/libref_grep.so"
