#!/bin/sh
# Build oracle/_ref/libqbref.so from the reference's own serial sources
# (Basis.cc, FourierTransform.cc with its internal FFT_NOLIB transform,
# UnitCell.cc, functionals/LDAFunctional.cc, the pseudopotential Species with
# its reader, radial sine transform, spherical integration and splines, and
# the vendored header-only XML parser), compiled in place from the read-only
# reference tree, plus the
# one-process Context stub and the C shim in this folder.  The reference's
# build system is not used.  Test infrastructure only.
#
#   build_ref.sh [REFERENCE_ROOT]     (or QBG_REFERENCE=REFERENCE_ROOT build_ref.sh)
#
# Without a reference root, or where its sources are absent, nothing is built.
set -e
REF=${1:-${QBG_REFERENCE:-}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ -z "$REF" ]; then
  echo "build_ref.sh: no reference root given (argument or QBG_REFERENCE); skipping" >&2
  exit 0
fi
if [ ! -f "$REF/src/qball/FourierTransform.cc" ]; then
  echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O2 -fPIC -shared -std=c++11 -w \
  -I"$HERE/ref_stub" -I"$REF/src" -I"$REF/src/qball" -I"$REF/src/functionals" \
  -I"$REF/external_libs/rapidxml" -DSHARE_DIR="\"$REF/share\"" \
  "$REF/src/qball/Basis.cc" "$REF/src/qball/FourierTransform.cc" \
  "$REF/src/qball/UnitCell.cc" "$REF/src/functionals/LDAFunctional.cc" \
  "$REF/src/qball/Species.cc" "$REF/src/qball/SpeciesReader.cc" \
  "$REF/src/qball/sinft.cc" "$REF/src/qball/SphericalIntegration.cc" \
  "$REF/src/pseudo/spline.cc" \
  "$HERE/ref_stub/ref_context_stub.cc" "$HERE/ref_shim.cc" \
  -o "$OUT/libqbref.so"
echo "built $OUT/libqbref.so"
