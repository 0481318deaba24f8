#!/usr/bin/env bash
# Build the reference fastmat (Cython) into baseline/_ref/ for use as a test
# oracle in this container only.  The reference tree is read-only, so it is
# copied first and two mechanical numpy-2 compatibility edits are applied to
# the copy:
#   1. np.NPY_NTYPES (removed in numpy 2) -> 24
#   2. np.NPY_{ENSURECOPY,OWNDATA,ENSUREARRAY,F_CONTIGUOUS,C_CONTIGUOUS}
#      -> np.NPY_ARRAY_* (the array-flag names numpy 2 keeps)
# Nothing produced here is committed (baseline/_ref/ is git-ignored) and
# nothing here runs on the GPU machine; the golden fixtures under
# tests/golden/ are what travels.
#
# Usage: oracle/build_reference.sh <path of the fastmat source tree>
#        (or FASTMAT_REFERENCE=<path> oracle/build_reference.sh)
set -euo pipefail
REF=${1:-${FASTMAT_REFERENCE:-}}
if [ -z "$REF" ] || [ ! -d "$REF/fastmat" ]; then
  echo "usage: $0 <fastmat source tree> (or set FASTMAT_REFERENCE)" >&2
  exit 2
fi
HERE=$(cd "$(dirname "$0")/.." && pwd)
DST="$HERE/baseline/_ref/src"
if [ -f "$DST/.built" ]; then echo "reference already built in $DST"; exit 0; fi
mkdir -p "$DST"
cp -r "$REF"/. "$DST"/
chmod -R u+w "$DST"
cd "$DST"
sed -i 's/np\.NPY_NTYPES/24/g' fastmat/core/types.pxd fastmat/core/types.pyx
for f in ENSURECOPY OWNDATA ENSUREARRAY F_CONTIGUOUS C_CONTIGUOUS; do
  sed -i "s/np\.NPY_${f}\b/np.NPY_ARRAY_${f}/g" fastmat/core/cmath.pyx
done
rm -f fastmat/*.c fastmat/core/*.c fastmat/algorithms/*.c
python3 setup.py build_ext --inplace -j 8 > "$HERE/baseline/_ref/build.log" 2>&1
python3 -c "import sys; sys.path.insert(0, '$DST'); import fastmat; print('fastmat', fastmat.__version__)"
touch "$DST/.built"
