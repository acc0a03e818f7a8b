#!/bin/bash
# Test infrastructure only: builds the reference's own CUDA sources, unmodified, into
# oracle/_ref/procell_ref for the distribution check (run on a machine with a GPU; it needs nvcc
# and links CUDA's device runtime for the reference's dynamic parallelism).
#
# Sources: /root/reference/src when mounted, else a copy placed in baseline/_ref/src
# (git-ignored) by `oracle/ref_build.sh --stage` on a machine that has /root/reference.
# The copy is never committed; it only travels with the working tree to the GPU machine.
# `--if-mounted` (used by the package build) builds from the mounted sources only, and only
# when the binary is missing or stale.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
OUT="$HERE/_ref"
if [[ "${1:-}" == "--stage" ]]; then
  mkdir -p "$ROOT/baseline/_ref"
  rm -rf "$ROOT/baseline/_ref/src"
  cp -r /root/reference/src "$ROOT/baseline/_ref/src"
  echo "staged reference sources in baseline/_ref/src"
  exit 0
fi
if [[ "${1:-}" == "--if-mounted" ]]; then
  # called by the package build: only where the reference is mounted, and only when the
  # binary is missing or older than the sources
  [[ -d /root/reference/src ]] || exit 0
  if [[ -x "$OUT/procell_ref" && -z "$(find /root/reference/src "$HERE/ref_compat.h" "$HERE/ref_timeshim.c" \
        -newer "$OUT/procell_ref" -print -quit)" ]]; then
    exit 0
  fi
fi
if [[ -d /root/reference/src ]]; then SRC=/root/reference/src; else SRC="$ROOT/baseline/_ref/src"; fi
[[ -d "$SRC" ]] || { echo "reference sources not found" >&2; exit 2; }
mkdir -p "$OUT/obj"
NVCC="${NVCC:-nvcc}"
FLAGS=(-O2 -std=c++17 -rdc=true -gencode arch=compute_103a,code=sm_103a -include "$HERE/ref_compat.h" -I "$SRC" -w)
FILES=(main.cu io/cmdargs.cpp io/parser.cu simulation/simulator.cu simulation/cells_population.cu
       simulation/cell.cu simulation/proliferation.cu utils/util.cu)
pids=()
for f in "${FILES[@]}"; do
  o="$OUT/obj/$(echo "$f" | tr '/.' '__').o"
  "$NVCC" "${FLAGS[@]}" -dc "$SRC/$f" -o "$o" & pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -gencode arch=compute_103a,code=sm_103a "$OUT"/obj/*.o -lcudadevrt -o "$OUT/procell_ref"
gcc -O2 -shared -fPIC "$HERE/ref_timeshim.c" -o "$OUT/libtimeshim.so"
echo "$OUT/procell_ref"
