#!/usr/bin/env bash
# Builds the unmodified reference implementation (s-cavalier/magnus-dp) as a
# CPU oracle: its pybind11 module `_core` plus its Python package, compiled
# straight from the reference's own source files (no CMake, no MKL, no JAX).
# Output goes only to oracle/_ref/ (git-ignored).  Nothing from the reference
# is copied into tracked files.
#
#   MAGNUS_REFERENCE   path of the reference checkout (default /root/reference)
#
# Recipe: generate the Gauss-Legendre table with the reference's own
# src/util/gen_nodes.py (order 64, the reference's CMake default), then one g++
# invocation over src/api/pybind.cpp, src/composer/backends.cpp,
# src/util/gausslegendre.cpp and the generated table.  The CBLAS calls of the
# Blas policy resolve to the naive header in oracle/ref_shim/mkl.h.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${MAGNUS_REFERENCE:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/magnus"
python3 "$REF/src/util/gen_nodes.py" 64 "$OUT/gl-nodes.cpp"
SUFFIX="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
PYBIND_INC="$(python3 -c 'import pybind11; print(pybind11.get_include())')"
PY_INC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
g++ -std=c++23 -O2 -fopenmp -fPIC -shared \
  -I "$REF/src" -I "$HERE/ref_shim" -I "$PYBIND_INC" -I "$PY_INC" \
  "$REF/src/api/pybind.cpp" "$REF/src/composer/backends.cpp" \
  "$REF/src/util/gausslegendre.cpp" "$OUT/gl-nodes.cpp" \
  -o "$OUT/magnus/_core$SUFFIX" -latomic
cp "$REF/src/api/magnus/__init__.py" "$OUT/magnus/__init__.py"
echo "built $OUT/magnus/_core$SUFFIX"
