#!/usr/bin/env bash
# Compile the reference's OpenCL kernels as C (test infrastructure only).
#
# Usage: TDE_REFERENCE=<reference checkout> bash oracle/build_ref.sh
#    or: bash oracle/build_ref.sh <reference checkout>
# Reads the read-only reference tree and writes one shared object per kernel
# into oracle/_ref/.  Nothing is copied out of the reference tree: gcc reads
# the .cl files where they lie.  The outputs are git-ignored.  Exit status 0
# with a message when no reference tree is given or found (machines without
# one run the tests on the committed golden vectors instead).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${TDE_REFERENCE:-}}"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -d "$REF/GPU/opencl" ]; then
    echo "build_ref: no reference tree (set TDE_REFERENCE or pass its path); skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
CFLAGS=(-std=gnu11 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -fvisibility=hidden
        -w -I "$REF/common/inc" -I "$REF/common/inc/types" -include "$HERE/ref_shim.h")
build() {  # <macro> <cl file> <output name>
    gcc "${CFLAGS[@]}" "-D$1" "-DREF_CL_PATH=\"$REF/GPU/opencl/$2\"" "$HERE/ref_launch.c" -o "$OUT/$3.so"
}
build REF_RAYCAST raycast.cl ref_raycast &
build REF_BILATERAL compute_bilateral_filtering.cl ref_bilateral &
build REF_TRANSFORM_MAP transform_map.cl ref_transform_map &
build REF_TRANSFORM_ESTIMATION transform_estimation.cl ref_transform_estimation &
build REF_CLEAN_BUFF clean_buff.cl ref_clean_buff &
build REF_SCAN_SLICE scan_slice_of_both_volumes.cl ref_scan_slice &
build REF_EXTRACT_SLICE extract_slice_as_cloud.cl ref_extract_slice &
build REF_CLEAN_COLOR_SLICE clean_color_slice.cl ref_clean_color_slice &
build REF_LSM compute_least_squares_equation.cl ref_lsm &
wait
ls "$OUT"
