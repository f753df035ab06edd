#!/bin/bash
# Builds the reference MACSIMUS `cook` variants used as the parity oracle and
# CPU baseline, straight from the reference sources with gcc (no makemake, no
# configure.sh).  Each variant gets its own simopt.h (compile-time switches,
# written here) and the module list that cook/configure.sh emits for the
# Ewald + linked-cell build.  Outputs go only to oracle/_ref/ (git-ignored).
#
# usage: oracle/build_ref.sh [REFERENCE_DIR]
# The reference tree is the argument, else $MACSIMUS_REF, else the read-only
# checkout this recipe was written against (/root/reference); without a
# reference tree the script does nothing and exits 0.
set -euo pipefail
REF=${1:-${MACSIMUS_REF:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
if [ ! -d "$REF/cook" ]; then
  echo "reference tree not found at $REF: skipping the reference build" >&2
  exit 0
fi
mkdir -p "$OUT"
# where the reference sources were found (read by the tests that compile
# against cook's headers)
echo "$REF" > "$OUT/REFERENCE_DIR"
# module list of cook/configure.sh (base list + "elst ewald linklist")
MODS="ground statics varfile bitfile cputime conjgrad gjlineq asksig simcg simgear \
interpot setss intrapot sitesite norm xforces linregr constrd rhs simglob pakcp \
simils siminit main simpot simmeas simmeasx forces simdef elst ewald linklist"
SRCS=""
for m in $MODS; do
  for d in gen sim sim/lj cook; do
    if [ -f "$REF/$d/$m.c" ]; then SRCS="$SRCS $REF/$d/$m.c"; break; fi
  done
done

variant() {  # name, extra libs, simopt lines...
  local name=$1; shift
  local libs=$1; shift
  local dir=$OUT/$name.d
  mkdir -p "$dir"
  {
    echo "#define COOK"
    echo "#define COULOMB -2"
    echo "#define SPLINE -2"
    echo "#define NONBOND \"lj\""
    echo "#define WORM"
    echo "#define LINKCELL 3"
    echo "#define VERLET 3"
    echo "#define SHAKE 1"
    for l in "$@"; do echo "$l"; done
    echo "#define PROJECT \"oracle-$name\""
  } > "$dir/simopt.h"
  if [ "$OUT/$name" -nt "$dir/simopt.h" ] && [ "$OUT/$name" -nt "$0" ]; then return 0; fi
  local objs=""
  for s in $SRCS; do
    local o=$dir/$(basename "$s" .c).o
    gcc -O2 -ffast-math -DSCR -w -I"$dir" -I"$REF/gen" -I"$REF/sim" -I"$REF/sim/lj" -I"$REF/cook" \
        -c "$s" -o "$o" &
    objs="$objs $o"
  done
  wait
  gcc -o "$OUT/$name" $objs -lm $libs
  echo "built $OUT/$name"
}

# serial Ewald + linked cells (the `cookewslc` configuration without SLAB)
variant cookew ""
# pthreads build (PARALLEL=1 + BARRIER): CPU baseline on all host cores
variant cookewP1 "-lpthread" "#define PARALLEL 1" "#define BARRIER"
# Drude polarizable build (POLAR=0: scalar linear polarizability)
variant cookpol "" "#define POLAR 0"
# Widom insertion build (WIDOM without SLAB)
variant cookwidom "" "#define WIDOM"
# full pressure tensor (PRESSURETENSOR = PT_VIR|PT_KIN|PT_OFF: virial and
# kinetic parts with the off-diagonal terms), plain and Drude builds
variant cookewpt "" "#define PRESSURETENSOR 7"
variant cookpolpt "" "#define POLAR 0" "#define PRESSURETENSOR 7"
