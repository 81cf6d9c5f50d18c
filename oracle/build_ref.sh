#!/usr/bin/env bash
# Compile the reference's own C++ extension (_skfn) from its sources where they
# lie, with g++ directly (no cmake), into oracle/_ref/.  Only used in the
# development container, where the reference checkout and pybind11 exist; the
# result validates the CPU oracle and generates tests/golden fixtures.
set -euo pipefail
REF=${SKFEM_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/cpp/src" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 0
fi
PYBIND_INC=$(python3 -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || true)
if [ -z "$PYBIND_INC" ]; then
  echo "pybind11 not importable; skipping reference build" >&2
  exit 0
fi
PY_INC=$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
EXT=$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
mkdir -p "$OUT/obj"
SRCS="bindings.cpp runtime.cpp assembly/linear_form_assembler.cpp assembly/functional_assembler.cpp \
assembly/supermesh_builder.cpp assembly/bilinear_form_assembler.cpp assembly/cross_bilinear_assembler.cpp \
assembly/cut_form_assembler.cpp assembly/cut_cross_assembler.cpp assembly/basis_geometry.cpp assembly/edge_topology.cpp"
pids=()
objs=()
for s in $SRCS; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$REF/cpp/src/$s" -nt "$o" ]; then
    g++ -std=c++17 -O3 -fPIC -fvisibility=hidden -I"$REF/cpp/include" -I"$PYBIND_INC" -I"$PY_INC" \
        -c "$REF/cpp/src/$s" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]:-}"; do [ -n "$p" ] && wait "$p"; done
g++ -shared -o "$OUT/_skfn$EXT" "${objs[@]}" -lpthread
echo "built $OUT/_skfn$EXT"
