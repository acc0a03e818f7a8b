#!/bin/bash
# Test infrastructure only: builds the reference's own CUDA sources, unmodified, for the
# distribution check and the timing comparison (run on a machine with a GPU; it needs nvcc
# and links CUDA's device runtime for the reference's dynamic parallelism). Two binaries:
#   oracle/_ref/procell_ref        sm_103a (the GB300's own architecture)
#   oracle/_ref/procell_ref_sm100  sm_100 only (the generic Blackwell build; its code runs
#                                   on the GB300 through binary compatibility within sm_10x)
#
# Sources: $PROCELL_REFERENCE_DIR/src (default /root/reference/src) when present, else a copy
# placed in baseline/_ref/src (git-ignored) by `oracle/ref_build.sh --stage` on a machine
# that has the reference. The copy is never committed; it only travels with the working tree
# to the GPU machine. `--if-mounted` (used by the package build) builds from the mounted
# sources only, and only when a binary is missing or stale.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
OUT="$HERE/_ref"
REFERENCE_DIR="${PROCELL_REFERENCE_DIR:-/root/reference}"
if [[ "${1:-}" == "--stage" ]]; then
  mkdir -p "$ROOT/baseline/_ref"
  rm -rf "$ROOT/baseline/_ref/src"
  cp -r "$REFERENCE_DIR/src" "$ROOT/baseline/_ref/src"
  echo "staged reference sources in baseline/_ref/src"
  exit 0
fi
if [[ "${1:-}" == "--if-mounted" ]]; then
  # called by the package build: only where the reference is mounted, and only when a
  # binary is missing or older than the sources
  [[ -d "$REFERENCE_DIR/src" ]] || exit 0
  stale=0
  for b in procell_ref procell_ref_sm100; do
    if [[ ! -x "$OUT/$b" || -n "$(find "$REFERENCE_DIR/src" "$HERE/ref_compat.h" "$HERE/ref_timeshim.c" \
          "$HERE/ref_build.sh" -newer "$OUT/$b" -print -quit)" ]]; then
      stale=1
    fi
  done
  [[ $stale == 1 ]] || exit 0
fi
if [[ -d "$REFERENCE_DIR/src" ]]; then SRC="$REFERENCE_DIR/src"; else SRC="$ROOT/baseline/_ref/src"; fi
[[ -d "$SRC" ]] || { echo "reference sources not found" >&2; exit 2; }
NVCC="${NVCC:-nvcc}"
FILES=(main.cu io/cmdargs.cpp io/parser.cu simulation/simulator.cu simulation/cells_population.cu
       simulation/cell.cu simulation/proliferation.cu utils/util.cu)
build() {  # build <binary name> <gencode>
  local name="$1" gencode="$2" obj="$OUT/obj_$1"
  mkdir -p "$obj"
  local pids=()
  for f in "${FILES[@]}"; do
    "$NVCC" -O2 -std=c++17 -rdc=true -gencode "$gencode" -include "$HERE/ref_compat.h" -I "$SRC" -w \
      -dc "$SRC/$f" -o "$obj/$(echo "$f" | tr '/.' '__').o" & pids+=($!)
  done
  for p in "${pids[@]}"; do wait "$p"; done
  "$NVCC" -gencode "$gencode" "$obj"/*.o -lcudadevrt -o "$OUT/$name"
}
mkdir -p "$OUT"
build procell_ref arch=compute_103a,code=sm_103a &
p1=$!
build procell_ref_sm100 arch=compute_100,code=sm_100 &
p2=$!
wait $p1
wait $p2
gcc -O2 -shared -fPIC "$HERE/ref_timeshim.c" -o "$OUT/libtimeshim.so"
echo "$OUT/procell_ref $OUT/procell_ref_sm100"
