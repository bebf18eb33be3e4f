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
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -eu
REF=${1:-/root/reference}
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
C
} > "$GEN"
${CC:-gcc} -O2 -shared -fPIC -o "$OUT/libref_grep.so" "$GEN"
echo "built $OUT/libref_grep.so"
