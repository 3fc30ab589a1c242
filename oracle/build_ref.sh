#!/usr/bin/env bash
# Builds the reference's own tracing kernels (unmodified, read in place from
# the reference checkout) as host shared objects under oracle/_ref/.
# Test infrastructure: the outputs are the oracle and the CPU baseline, never
# part of the fastqsl_gb300 package.  Needs the reference checkout, so it runs
# only where that exists; elsewhere oracle/build.py skips it.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]      (default /root/reference)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference}"
cu="$ref/fastqslpy/cu"
out="$here/_ref"
cuda_inc="${CUDA_HOME:-/usr/local/cuda}/include"
if [ ! -f "$cu/TraceBlineAdaptive.cu" ]; then
    echo "reference kernels not found under $cu" >&2
    exit 3
fi
mkdir -p "$out"
# -ffp-contract=off: no fused multiply-add, so every float operation rounds
# exactly as written (the same rule the oracle restatement is built with).
flags=(-O2 -std=c++17 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math
       -fvisibility=hidden -w -I "$here/ref_shim" -I "$cu" -I "$cuda_inc"
       -Wl,--version-script="$here/ref_shim/exports.map")
pids=()
for k in 1 2 3 4; do
    name=(x rk4 rkf45 scott stretch)
    g++ "${flags[@]}" -DREF_KERNEL=$k "$here/ref_shim/ref_driver.cpp" -o "$out/libqslref_${name[$k]}.so" &
    pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
