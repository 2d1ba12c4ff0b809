#!/usr/bin/env bash
# Builds the unmodified reference implementation (s-cavalier/magnus-dp) as a
# CPU oracle: its pybind11 module `_core` plus its Python package, compiled
# straight from the reference's own source files (no CMake, no MKL, no JAX).
# Output goes only to oracle/_ref/ (git-ignored).  Nothing from the reference
# is copied into tracked files.
#
#   MAGNUS_REFERENCE   path of the reference checkout (default: a checkout
#                      named `reference` beside this repository)
#
# Recipe: generate the Gauss-Legendre table with the reference's own
# src/util/gen_nodes.py (order 64, the reference's CMake default), then one g++
# invocation over src/api/pybind.cpp, src/composer/backends.cpp,
# src/util/gausslegendre.cpp and the generated table.  The CBLAS calls of the
# Blas policy resolve to the naive header in oracle/ref_shim/mkl.h.
#
# Second module (when the engine's libmagnus_gb300.so is built): the same
# sources with the "GB300" matrix backend bound in (ref_gb300/patch_pybind.py
# writes the patched pybind.cpp into oracle/_ref/gb300/, ref_gb300/
# gb300_backend.hpp holds the routing bodies), linked against the engine, as
# oracle/_ref/gb300/magnus/_core: the reference's own Python API with
# matrix_backend="GB300".
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
REF="${MAGNUS_REFERENCE:-$(cd "$ROOT/.." && pwd)/reference}"
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
CORE="$OUT/magnus/_core$SUFFIX"
if [ ! -f "$CORE" ]; then
  g++ -std=c++23 -O2 -fopenmp -fPIC -shared \
    -I "$REF/src" -I "$HERE/ref_shim" -I "$PYBIND_INC" -I "$PY_INC" \
    "$REF/src/api/pybind.cpp" "$REF/src/composer/backends.cpp" \
    "$REF/src/util/gausslegendre.cpp" "$OUT/gl-nodes.cpp" \
    -o "$CORE" -latomic
  cp "$REF/src/api/magnus/__init__.py" "$OUT/magnus/__init__.py"
  echo "built $CORE"
fi

LIBDIR="$ROOT/magnus-dp_gb300/magnus_gb300"
if [ -f "$LIBDIR/libmagnus_gb300.so" ]; then
  G="$OUT/gb300"
  mkdir -p "$G/magnus"
  python3 "$HERE/ref_gb300/patch_pybind.py" "$REF/src/api/pybind.cpp" "$G/pybind_gb300.cpp"
  g++ -std=c++23 -O2 -fopenmp -fPIC -shared \
    -I "$REF/src" -I "$HERE/ref_shim" -I "$HERE/ref_gb300" -I "$ROOT/include" -I "$PYBIND_INC" -I "$PY_INC" \
    "$G/pybind_gb300.cpp" "$REF/src/composer/backends.cpp" \
    "$REF/src/util/gausslegendre.cpp" "$OUT/gl-nodes.cpp" \
    -o "$G/magnus/_core$SUFFIX" -L "$LIBDIR" -lmagnus_gb300 -Wl,-rpath,"$LIBDIR" -latomic
  cp "$REF/src/api/magnus/__init__.py" "$G/magnus/__init__.py"
  echo "built $G/magnus/_core$SUFFIX (matrix_backend=\"GB300\" bound to libmagnus_gb300.so)"
fi
