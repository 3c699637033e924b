#!/usr/bin/env bash
# Build the project's CPU restatement (test oracle) into oracle/liborc.so.
# Plain C, portable (no -march=native): it runs on x86 here and on Arm hosts.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
CC="${CC:-gcc}"
"$CC" -O3 -std=c99 -fPIC -shared -Wall -Wno-unused-function -o "$HERE/liborc.so" \
  "$HERE/igap_oracle.c" "$HERE/laws.c" "$HERE/law_gradelast.c" "$HERE/law_lingrad.c" -lm
echo "build_oracle: built $HERE/liborc.so"
