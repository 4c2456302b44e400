#!/usr/bin/env bash
# Builds oracle/_ref/libref_harness.so from the reference sources where they
# lie (default /root/reference; override with REF_ROOT).  Oracle
# infrastructure: used only to pin the CPU restatement and to generate the
# golden fixtures in tests/golden/.  The reference's own CMake build is not
# used; the flags below restate src/CMakeLists.txt:19-22 (BIASED_SAMPLING),
# without GL_SIMD: its SIMD path reads uninitialised vector lanes
# (include/utils/matrix.hpp:255,458), so the scalar path is the defined one.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
OUT="$REPO/oracle/_ref"
if [ ! -d "$REF_ROOT/include" ]; then
  echo "reference sources not found at $REF_ROOT; skipping reference harness" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
SHIM="$HERE/shim"
FLAGS=(-std=c++17 -O2 -fPIC -ffp-contract=off -DBIASED_SAMPLING -w
       -include "$SHIM/ref_compat.hpp" -include "$SHIM/ref_rng.hpp")
case "$(uname -m)" in
  x86_64) FLAGS+=(-iquote "$SHIM") ;;   # sse2neon.h is ARM-only: use <immintrin.h>
esac
FLAGS+=(-I"$REF_ROOT/include" -I"$REF_ROOT/src")
SRCS=(material/disneyPrincipledBSDF material/hairMarsch primitives/meshBVH
      primitives/triangleMesh base/primitive base/object3D base/framebuffer
      base/camera base/objectList sampler/sampler texture/texture
      utils/objectTransform PDF/hairPDF mesh_io/meshLoader mesh_io/fbxLoader)
pids=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr / _).o"
  g++ "${FLAGS[@]}" -c "$REF_ROOT/src/$s.cpp" -o "$o" & pids+=($!)
done
g++ "${FLAGS[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" & pids+=($!)
g++ "${FLAGS[@]}" -c "$SHIM/ref_rng.cpp" -o "$OUT/obj/ref_rng.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libref_harness.so" "$OUT"/obj/*.o -lpthread
# where the harness was built from (tests read the reference's own files there)
printf '%s\n' "$REF_ROOT" > "$OUT/REF_ROOT"
echo "built $OUT/libref_harness.so"
