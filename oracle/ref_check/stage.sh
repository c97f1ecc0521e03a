#!/bin/sh
# Stages the reference's hot-path sources for the cross-check build: copies the
# reference checkout's top-level headers, main.cpp and settings/*.ini from
# REF_SRC (default: the checkout at /root/reference on the build machine) into
# baseline/_ref/, the git-ignored location of the reference install.  Nothing
# staged is committed; the copy travels with the working tree to a machine
# without the checkout, where oracle/ref_check/build.sh compiles it in place.
# Exits 2 (nothing copied) when the checkout is absent.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
SRC="${REF_SRC:-/root/reference}"
DST="$REPO/baseline/_ref"
[ -f "$SRC/Update.h" ] || { echo "reference checkout not found at $SRC" >&2; exit 2; }
mkdir -p "$DST/settings"
cp "$SRC"/*.h "$SRC/main.cpp" "$DST/"
cp "$SRC"/settings/*.ini "$DST/settings/"
echo "staged the reference sources in $DST"
