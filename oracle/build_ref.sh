#!/usr/bin/env bash
# Builds HEAL's own sample implementation (example_impl + py_bindings) from
# the reference sources where they lie, into oracle/_ref/ (git-ignored).
# The reference location is the first argument, else HEAL_REFERENCE, else
# the development container's checkout (oracle/reference.py finds the same).
# Used only in the development container to pin the oracle and to write the
# golden fixtures under tests/golden/; the GPU host never has the sources.
# The reference's CMake forces _GLIBCXX_USE_CXX11_ABI=0 (CMakeLists.txt:11),
# which does not match the installed torch, so it is compiled directly here.
set -euo pipefail
REF=${1:-${HEAL_REFERENCE:-/root/reference}}
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
[ -d "$REF/example_impl" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
TORCH=$(python3 -c "import torch,os;print(os.path.dirname(torch.__file__))")
PYINC=$(python3 -c "import sysconfig;print(sysconfig.get_paths()['include'])")
SUFFIX=$(python3 -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
CXXFLAGS="-std=c++17 -O2 -fopenmp -fPIC -I$REF/include -I$REF/example_impl -I$TORCH/include -I$TORCH/include/torch/csrc/api/include -I$PYINC"
pids=()
for f in "$REF"/example_impl/*_impl.cpp "$REF"/example_impl/py_bindings.cpp; do
  o="$OUT/$(basename "${f%.cpp}").o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then g++ $CXXFLAGS -c "$f" -o "$o" & pids+=($!); fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/lattica_hw$SUFFIX" "$OUT"/*.o -L"$TORCH/lib" -Wl,-rpath,"$TORCH/lib" \
    -ltorch -ltorch_cpu -lc10 -ltorch_python
echo "built $OUT/lattica_hw$SUFFIX"
