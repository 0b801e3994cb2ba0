#!/usr/bin/env bash
# Builds the reference solver's own search code for the CPU into oracle/_ref/
# (test infrastructure only; the output is git-ignored and never shipped).
#
# The sources are compiled where they lie under the reference checkout; none
# is copied.  The only transformation is done on the fly by sed: the CUDA
# launch syntax `<<<grid, block, smem, stream>>>` on solver.cu:331 (and
# thinker.cu:374) is removed, which turns BatchedTask::launch into a direct
# call of alpha_beta_kernel on the host (BatchedThinkTask::launch of
# think_kernel likewise; see refshim/prelude.h for the single-thread
# mapping).  board.cu is compiled with __CUDA_ARCH__ defined so that its
# device branch (the code the GPU runs) is emulated rather than its host
# branch, whose __builtin_clzll(0) is undefined and gives wrong flips when a
# ray holds only opponent discs.
# to_board.cpp uses SSSE3/SSE4.1 intrinsics, so this recipe only builds on
# x86-64; on other hosts it exits 0 without building anything.
set -euo pipefail
REF="${REF:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/solver.cu" ]; then
  echo "ref_build: no reference checkout at $REF; skipped" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64) ;;
  *) echo "ref_build: reference codec needs x86-64 SSE4.1; skipped" >&2; exit 0 ;;
esac
mkdir -p "$OUT"
CXX="${CXX:-g++}"
EMU=("$CXX" -std=c++17 -O2 -include "$HERE/refshim/prelude.h" -I "$HERE/refshim" -I "$REF" -x c++)
sed -e 's/<<<[^>]*>>>//' "$REF/solver.cu" | "${EMU[@]}" -c - -o "$OUT/solver.o" &
"${EMU[@]}" -D__CUDA_ARCH__=1030 -c "$REF/board.cu" -o "$OUT/board.o" &
"${EMU[@]}" -c "$REF/table.cu" -o "$OUT/table.o" &
"$CXX" -std=c++17 -O2 -msse4.1 -I "$REF" -c "$REF/to_board.cpp" -o "$OUT/to_board.o" &
"${EMU[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" &
"$CXX" -std=c++17 -O2 -msse4.1 -I "$REF" -c "$REF/test.cpp" -o "$OUT/test.o" &
# think mode: the launch on thinker.cu:374-375 is removed the same way, and
# eval.cu runs its device branch (software bit extract, no x86 pext)
sed -e 's/<<<[^>]*>>>//' "$REF/thinker.cu" | "${EMU[@]}" -c - -o "$OUT/thinker.o" &
"${EMU[@]}" -D__CUDA_ARCH__=1030 -c "$REF/eval.cu" -o "$OUT/eval.o" &
"${EMU[@]}" -c "$HERE/ref_think_harness.cpp" -o "$OUT/ref_think_harness.o" &
wait
"$CXX" -o "$OUT/refsolve" "$OUT/ref_harness.o" "$OUT/solver.o" "$OUT/board.o" "$OUT/table.o" "$OUT/to_board.o"
"$CXX" -o "$OUT/reftest" "$OUT/test.o" "$OUT/to_board.o"
"$CXX" -o "$OUT/refthink" "$OUT/ref_think_harness.o" "$OUT/thinker.o" "$OUT/eval.o" \
    "$OUT/board.o" "$OUT/table.o" "$OUT/to_board.o"
echo "ref_build: built $OUT/refsolve, $OUT/refthink and $OUT/reftest" >&2
