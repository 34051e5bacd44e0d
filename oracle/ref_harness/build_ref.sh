#!/usr/bin/env bash
# Builds the reference's own FP64 cuFFT stepper plus the step-by-step harness
# (harness.cpp) into oracle/_ref/refstep.  TEST INFRASTRUCTURE ONLY.
#
# Sources: the reference tree given by $CB_REFERENCE_SRC (default: a directory
# named "reference" beside the repository).  When that tree exists, the needed files are staged,
# unmodified, into oracle/_ref/src/ (git-ignored) so that a machine without
# the reference tree (the GPU host) can rebuild from the staged copy.  No
# reference file is edited: CUDA-13 API drift is absorbed by the forced-include
# shim refshim.h.  Outputs go only to oracle/_ref/.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(cd "$here/../.." && pwd)"
out="$root/oracle/_ref"
src="$out/src"
ref="${CB_REFERENCE_SRC:-$root/../reference}"
files="Calc.cu Calc.h belastic.cpp belastic.h fluidbase.cpp fluidbase.h phasefield.cpp phasefield.h
       tool.cpp tool.cu tool.h mem_array.cpp mem_array.h stdafx.h drawbubble.cpp stb_image.h
       stb_image_write.h stb_image_resize.h"
mkdir -p "$src" "$out/obj" "$out/inc/sys"
if [ -d "$ref" ]; then
  for f in $files; do cp -f "$ref/$f" "$src/$f"; done
fi
for f in $files; do
  [ -f "$src/$f" ] || { echo "build_ref: missing $src/$f (no reference tree to stage from)" >&2; exit 3; }
done
# glibc >= 2.33 no longer ships <sys/timeb.h>, which stdafx.h includes but
# never uses; an empty stand-in keeps the include line valid.
[ -f /usr/include/sys/timeb.h ] || : > "$out/inc/sys/timeb.h"

NVCC="${NVCC:-nvcc}"
ARCH="-gencode arch=compute_103a,code=sm_103a"
DEFS="-Dprivate=public -Dprotected=public"
FLAGS="-O2 -std=c++14 -w $ARCH $DEFS -I$src -I$out/inc"
pids=()
compile() {  # $1 source, $2 object, rest extra flags
  local s="$1" o="$2"; shift 2
  "$NVCC" $FLAGS "$@" -c "$s" -o "$o"
}
compile "$src/Calc.cu" "$out/obj/Calc.o" -include "$here/refshim.h" & pids+=($!)
compile "$src/tool.cu" "$out/obj/tool_cu.o" & pids+=($!)
for f in belastic fluidbase phasefield tool mem_array drawbubble; do
  compile "$src/$f.cpp" "$out/obj/$f.o" -x cu & pids+=($!)
done
compile "$here/harness.cpp" "$out/obj/harness.o" -x cu & pids+=($!)
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc -eq 0 ] || { echo "build_ref: compile failed" >&2; exit 1; }
"$NVCC" $ARCH "$out"/obj/*.o -o "$out/refstep" -lcufft
echo "build_ref: built $out/refstep"
