#!/usr/bin/env bash
# Builds the reference's own 3D eikonal entry point (fastMarching3D) from its
# C++ sources where they lie, with the project's Boost heap stand-in, into
# oracle/_ref/libfmm_ref.so. Test infrastructure only: used to pin the
# oracle's restatement (oracle/sfmm3d.cpp) and as the CPU reference baseline.
# Flags follow the reference makefile (src/makefile: -O3 -std=c++11
# -frounding-math); -ffp-contract=off keeps FMA contraction off on every host.
set -euo pipefail
REF=${MCT_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
FM="$REF/fastmarching"
if [ ! -f "$FM/fastMarching.cpp" ]; then
  echo "reference sources not found at $FM (set MCT_REFERENCE)" >&2
  exit 2
fi
mkdir -p "$HERE/_ref"
g++ -O3 -std=c++11 -frounding-math -ffp-contract=off -fPIC -shared -w \
  -I"$HERE/boost_shim" -I"$FM" -I"$FM/console" -I"$FM/ndgridmap" -I"$FM/fmm" \
  -I"$FM/fmm/fmdata" -I"$FM/io" -I"$FM/gradientdescent" \
  "$FM/fastMarching.cpp" "$FM/console/console.cpp" "$FM/ndgridmap/cell.cpp" \
  "$FM/fmm/fmdata/fmcell.cpp" -o "$HERE/_ref/libfmm_ref.so"
echo "built $HERE/_ref/libfmm_ref.so"
