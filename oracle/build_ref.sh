#!/usr/bin/env bash
# Builds the reference's own NRG engine as the CPU oracle (oracle/_ref/ref_nrg).
# The reference headers are compiled unchanged from where they lie; LAPACKE and
# CBLAS calls are routed to scipy's bundled OpenBLAS through oracle/shim/.
# Needs the reference tree (default /root/reference, override with NRG_REF_ROOT);
# exits 0 without building when it is absent (the GPU host has no copy).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${NRG_REF_ROOT:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/nrgcore/include/nrgcore/nrgcore.hpp" ]; then
  echo "build_ref: reference tree not found at $REF; skipping" >&2
  exit 0
fi
BLAS="$(python3 - <<'PY'
import glob, os, scipy
d = os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs")
c = sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so")))
print(os.path.realpath(c[0]) if c else "")
PY
)"
if [ -z "$BLAS" ]; then echo "build_ref: scipy OpenBLAS not found" >&2; exit 1; fi
mkdir -p "$OUT"
if [ -x "$OUT/ref_nrg" ] && [ -z "$(find "$HERE/drivers" "$HERE/shim" "$HERE/build_ref.sh" -newer "$OUT/ref_nrg" -print -quit)" ]; then
  echo "build_ref: $OUT/ref_nrg is up to date"
  exit 0
fi
g++ -std=c++20 -O3 -fopenmp -w \
  -I"$HERE/shim" -I"$REF/nrgcore/include" \
  "$HERE/drivers/ref_nrg.cpp" "$REF/nrgcore/src/models/twoChannel.cpp" \
  -o "$OUT/ref_nrg" "$BLAS" -Wl,-rpath,"$(dirname "$BLAS")"
echo "built $OUT/ref_nrg"
