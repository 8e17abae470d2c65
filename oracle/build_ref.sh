#!/usr/bin/env bash
# Builds oracle/_ref/libsr_ref.so: the reference's own far- and near-field
# OpenCL kernels (synchrad/kernel_farfield.cl, synchrad/kernel_nearfield.cl),
# compiled as C++ for the CPU through oracle/ref_shim.hpp and driven by
# oracle/ref_driver.cpp.
#
# TEST INFRASTRUCTURE ONLY.  The Mako placeholders are substituted the way
# synchrad/calc.py:610-616 does it (${my_dtype} -> double|float,
# ${f_native} -> '').  The substituted text goes straight into g++ through a
# pipe: no copy of the reference source is written anywhere.  The only outputs
# are the object files and the library under oracle/_ref/ (git-ignored).
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-/root/reference}"
OUT="$HERE/_ref"
CXX="${CXX:-g++}"
CXXFLAGS=(-std=gnu++17 -O2 -fPIC -ffp-contract=off -fopenmp -w)

if [[ ! -f "$REF/synchrad/kernel_farfield.cl" ]]; then
  echo "build_ref.sh: reference kernels not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"

compile_kernel() {  # $1 = far|near, $2 = double|float
  local mode="$1" dtype="$2"
  local src="$REF/synchrad/kernel_${mode}field.cl"
  {
    echo "namespace sr_ref_${mode}_${dtype} {"
    sed -e "s/\${my_dtype}/${dtype}/g" -e "s/\${f_native}//g" \
        -e '/#pragma OPENCL/d' "$src"
    echo "}"
  } | "$CXX" "${CXXFLAGS[@]}" -include "$HERE/ref_shim.hpp" -x c++ -c - \
        -o "$OUT/${mode}_${dtype}.o"
}

for mode in far near; do
  for dtype in double float; do
    compile_kernel "$mode" "$dtype"
  done
done
"$CXX" "${CXXFLAGS[@]}" -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o"
"$CXX" -shared -fopenmp -o "$OUT/libsr_ref.so" "$OUT/ref_driver.o" \
  "$OUT/far_double.o" "$OUT/far_float.o" "$OUT/near_double.o" \
  "$OUT/near_float.o"
echo "built $OUT/libsr_ref.so"
