#!/usr/bin/env bash
# Compile the reference's own assembly path, UNCHANGED from its source tree,
# against the project's single-rank MPI/PETSc stand-ins, into
# oracle/_ref/libigapref.so (git-ignored).  Test infrastructure only.
#
# Reads the reference tree at IGAP4_REF (default /root/reference, where the
# tree is mounted in the build container).  Where it is absent (e.g. on a
# machine without the reference) this script exits 0 without building, and the
# tests use the golden fixtures and the project's own C restatement
# (oracle/liborc.so, built by build_oracle.sh).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${IGAP4_REF:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/assmcore_iga.c" ]; then
  echo "build_ref: reference sources not found at $REF; skipping"
  exit 0
fi
mkdir -p "$OUT"
CC="${CC:-gcc}"
# -std=c99 as in the reference makefile; no -march=native so the oracle is
# portable; -O2 keeps the C99 'inline' helpers of include/mathutil.h inlined.
CFLAGS="-O2 -std=c99 -fPIC -w -I$HERE/stub -I$REF/include"
SRCS=(
  "$REF/src/assmcore_iga.c" "$REF/src/meshcore_iga.c" "$REF/src/commcore_iga.c"
  "$REF/src/postcore_iga.c" "$REF/src/ioutil.c" "$REF/src/interface.c"
  "$REF/src/quadrature.c" "$REF/src/mathutil.c"
  "$REF/mesh/igabeam.c" "$REF/mesh/meshigabeam.c"
  "$REF/mesh/igabeamtest.c" "$REF/mesh/meshigabeamtest.c"
  "$REF/phys/gradelast.c" "$REF/phys/physgradelast.c"
  "$REF/phys/gradelasttime.c" "$REF/phys/physgradelasttime.c"
  "$HERE/stub/stub_impl.c" "$HERE/ref_driver.c" "$HERE/law_lingrad.c"
)
OBJDIR="$OUT/obj"
mkdir -p "$OBJDIR"
pids=()
objs=()
for s in "${SRCS[@]}"; do
  o="$OBJDIR/$(basename "$(dirname "$s")")_$(basename "$s" .c).o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then
    "$CC" $CFLAGS -c "$s" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CC" -shared -o "$OUT/libigapref.so" "${objs[@]}" -lm
echo "build_ref: built $OUT/libigapref.so"
