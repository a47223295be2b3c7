#!/bin/sh
# Writes tests/golden/paramvar_layout.json: sizeof/offsetof of every member
# of the reference's paramVar (typeDefinition.cuh:35-125), measured by
# compiling the reference header with nvcc (host code only, no GPU needed).
# Runs where the reference sources are mounted; the JSON is committed.
set -e
REF=${YH_REFERENCE:-/root/reference}
here=$(cd "$(dirname "$0")" && pwd)
tmp=$(mktemp -d)
fields=$(python3 -c "
import sys; sys.path.insert(0, '$here/../..')
from yolohtli_gb300._abi import PARAM_FIELD_NAMES
print(' '.join(PARAM_FIELD_NAMES))")
{
  echo '#include <cstdio>'
  echo '#include <cstddef>'
  echo "#include \"$REF/typeDefinition.cuh\""
  echo 'int main() {'
  echo '  std::printf("{\"sizeof\": %zu, \"offsets\": {", sizeof(paramVar));'
  sep=""
  for f in $fields; do
    echo "  std::printf(\"$sep\\\"$f\\\": %zu\", offsetof(paramVar, $f));"
    sep=", "
  done
  echo '  std::printf("}}\\n");'
  echo '}'
} > "$tmp/layout.cu"
nvcc -x cu "$tmp/layout.cu" -o "$tmp/layout"
"$tmp/layout" > "$here/paramvar_layout.json"
rm -rf "$tmp"
