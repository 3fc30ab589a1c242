#!/usr/bin/env bash
# Builds the reference's own tracing kernels (read in place from the
# reference checkout; one line of TraceBlineScott.cu changed in a copy, see
# below) as host shared objects under oracle/_ref/.
# Test infrastructure: the outputs are the oracle and the CPU baseline, never
# part of the fastqsl_gb300 package.  Needs the reference checkout, so it runs
# only where that exists; elsewhere oracle/build.py skips it.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]
#
# REFERENCE_ROOT defaults to $QSL_REFERENCE_ROOT, else to a directory named
# `reference` beside this repository.
#
# TraceBlineScott.cu is compiled from a copy written to oracle/_ref/ at build
# time with one line changed: the tolerance it reads uninitialised
# (TraceBlineScott.cu:352,378, `tol_this=tol_this*tol_coef;`) becomes
# `tol_this=TOL*tol_coef;` (its TOL macro, 1e-3, times the caller's
# coefficient).  As shipped, the host build of the whole-line routine reads
# stack garbage there (a crash or an arbitrary tolerance); with the change it
# runs, and its per-step functions are the unmodified ones.  Nothing else in
# the copy differs; the copy is never committed.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${QSL_REFERENCE_ROOT:-$here/../../reference}}"
cu="$ref/fastqslpy/cu"
out="$here/_ref"
cuda_inc="${CUDA_HOME:-/usr/local/cuda}/include"
if [ ! -f "$cu/TraceBlineAdaptive.cu" ]; then
    echo "reference kernels not found under $cu" >&2
    exit 3
fi
mkdir -p "$out"
# the Scott kernel with its tolerance initialised (see above)
mkdir -p "$out/scott_tolfix"
sed 's/tol_this=tol_this\*tol_coef;/tol_this=TOL*tol_coef;/' "$cu/TraceBlineScott.cu" > "$out/scott_tolfix/TraceBlineScott.cu"
if [ "$(grep -c 'tol_this=TOL\*tol_coef;' "$out/scott_tolfix/TraceBlineScott.cu")" != 1 ] ||
   [ "$(diff "$cu/TraceBlineScott.cu" "$out/scott_tolfix/TraceBlineScott.cu" | grep -c '^[<>]')" != 2 ]; then
    echo "TraceBlineScott.cu: the tolerance line was not found exactly once" >&2
    exit 4
fi
# -ffp-contract=off: no fused multiply-add, so every float operation rounds
# exactly as written (the same rule the oracle restatement is built with).
flags=(-O2 -std=c++17 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math
       -fvisibility=hidden -w -I "$here/ref_shim" -I "$cu" -I "$cuda_inc"
       -Wl,--version-script="$here/ref_shim/exports.map")
pids=()
for k in 1 2 3 4; do
    name=(x rk4 rkf45 scott stretch)
    extra=()
    if [ "$k" = 3 ]; then extra=(-I "$out/scott_tolfix"); fi
    g++ "${extra[@]}" "${flags[@]}" -DREF_KERNEL=$k "$here/ref_shim/ref_driver.cpp" -o "$out/libqslref_${name[$k]}.so" &
    pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
