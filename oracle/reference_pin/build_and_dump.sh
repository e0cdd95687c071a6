#!/bin/sh
# Build the unmodified reference (its src/*.cpp but main.cpp and tests.cpp)
# with dump_reference.cpp against an installed SEAL 4.1 -- the fork the
# reference names in README.md:11-18 (it provides prepare_seeded_gsw_key),
# built without HEXL -- and dump one query's arrays for
# tests/test_reference_dump.py.  Nothing is fetched: SEAL must be supplied.
#
#   SEAL_PREFIX=/path/to/seal/install [REFERENCE=/path/to/OnionPIRv2] \
#     [PIN_PRESET=n4096] oracle/reference_pin/build_and_dump.sh [OUT_DIR]
#
# OUT_DIR defaults to oracle/_ref/dump (or oracle/_ref/dump_n4096); the tests
# read it from there, or from $OPIR_REFERENCE_DUMP.
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
REF=${REFERENCE:-/root/reference}
: "${SEAL_PREFIX:?set SEAL_PREFIX to a SEAL 4.1 (OnionPIR fork) install prefix}"
SEAL_INC=$(ls -d "$SEAL_PREFIX"/include/SEAL-4.* | head -1)
SEAL_LIB=$(ls "$SEAL_PREFIX"/lib*/libseal*.a "$SEAL_PREFIX"/lib*/libseal*.so 2>/dev/null | head -1)
DEFS=""
OUT_DEFAULT="$ROOT/oracle/_ref/dump"
if [ "${PIN_PRESET:-}" = "n4096" ]; then
  DEFS="-DPIN_N4096"
  OUT_DEFAULT="$ROOT/oracle/_ref/dump_n4096"
fi
OUT=${1:-$OUT_DEFAULT}
mkdir -p "$ROOT/oracle/_ref" "$OUT"
SRCS=""
for f in "$REF"/src/*.cpp; do
  case "$(basename "$f")" in main.cpp | tests.cpp) ;; *) SRCS="$SRCS $f" ;; esac
done
# this directory first: its database_constants.h selects the dumped preset
g++ -std=c++20 -O2 $DEFS -I "$HERE" -I "$REF/src/includes" -I "$SEAL_INC" \
  $SRCS "$HERE/dump_reference.cpp" "$SEAL_LIB" -lpthread -o "$ROOT/oracle/_ref/dump_reference"
"$ROOT/oracle/_ref/dump_reference" "$OUT" 1234
