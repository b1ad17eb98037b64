#!/bin/sh
# Builds oracle/_ref/libfpl_ref.so: the oracle's per-pixel loop linked to the
# reference's own EVWorker (include/fringe/EigenLapack.hpp), compiled from the
# reference tree where it lies, with LAPACK taken from SciPy's bundled
# OpenBLAS (its symbols carry a "scipy_" prefix).  Test infrastructure only.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#        oracle/build_ref.sh --root     (prints the reference tree it would use)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
if [ "$1" = "--root" ]; then
    echo "${FRINGE_REFERENCE_ROOT:-/root/reference}"
    exit 0
fi
REF=${1:-${FRINGE_REFERENCE_ROOT:-/root/reference}}
if [ ! -f "$REF/include/fringe/EigenLapack.hpp" ]; then
    echo "build_ref: reference headers not found under $REF; skipping" >&2
    exit 3
fi
SCIPY_LIBS=$(python3 -c "import scipy, os; print(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), 'scipy.libs'))")
OPENBLAS=$(ls "$SCIPY_LIBS"/libscipy_openblas*.so 2>/dev/null | head -1)
if [ -z "$OPENBLAS" ]; then
    echo "build_ref: no SciPy OpenBLAS found in $SCIPY_LIBS; skipping" >&2
    exit 3
fi
mkdir -p "$HERE/_ref"
LAPACK_DEFS="-Dzheevr_=scipy_zheevr_ -Dzpotrf_=scipy_zpotrf_ -Dzpotri_=scipy_zpotri_"
gcc -O2 -fPIC -fopenmp -ffp-contract=off -fcx-limited-range -DFPL_BACKEND_REF \
    -c "$HERE/fpl_oracle.c" -o "$HERE/_ref/fpl_oracle_ref.o"
gcc -O2 -fPIC -fopenmp -ffp-contract=off -fcx-limited-range -DFPL_BACKEND_REF \
    -c "$HERE/fpl_nmap_oracle.c" -o "$HERE/_ref/fpl_nmap_oracle_ref.o"
g++ -O2 -fPIC -std=c++11 $LAPACK_DEFS -I"$REF/include" -I"$REF/src/nmap" \
    -c "$HERE/ref_backend.cpp" -o "$HERE/_ref/ref_backend.o"
g++ -shared -fopenmp -o "$HERE/_ref/libfpl_ref.so" \
    "$HERE/_ref/fpl_oracle_ref.o" "$HERE/_ref/fpl_nmap_oracle_ref.o" "$HERE/_ref/ref_backend.o" \
    -L"$SCIPY_LIBS" -l:$(basename "$OPENBLAS") -Wl,-rpath,"$SCIPY_LIBS"
rm -f "$HERE/_ref/fpl_oracle_ref.o" "$HERE/_ref/fpl_nmap_oracle_ref.o" "$HERE/_ref/ref_backend.o"
echo "built $HERE/_ref/libfpl_ref.so (LAPACK: $(basename "$OPENBLAS"))"
