#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.  Compiles the reference's own OSTR code for the CPU
# into oracle/_ref/libostr_ref.so, straight from the reference sources where
# they lie (nothing is copied into this repository):
#   Tomo_OSTR.cu       18-116  host globals and __constant__ geometry
#                     118-325  G_Q2_prior, G_Fessler_prior, G_Huber_prior
#                     327-610  Siddon device function of the SART projector
#                     612-1173 Siddon device functions (OSTR, normprj)
#                    1177-1311 SART projector kernels (plain and _cos)
#                    1313-1449 OSTR_cos and normprj kernels
#                    1453-1515 the 4R sub-ray kernel (its undefined batch counts
#                              come from ref/ref_shim.h; the merge kernel
#                              :1517-1550 reads an unassigned index and is left out)
#                    1553-1735 backprj_gpu_manyviews_SBP
#                    1737-2183 backprj_OSSART{,_R}_gpu_manyviews, SART_prj_diff_kernel
#   Tomo_OSTR_gold.cpp 22-1528 I/O, compute_yry/h, regroup, update_est,
#                              both OSTR drivers, import_param, Reconstruction
# The rest of Tomo_OSTR.cu (the 4R merge kernel, launch wrappers with
# <<< >>>, main) is left out; ref/ref_launch.inc stands in for the
# launch wrappers.  Tomo_OSTR.h / readdata.h /
# helper_cuda.h are absent from the reference, so their includes (the first
# lines of each file) are skipped.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# the reference sources: NR_REFERENCE_DIR, else a checkout named "reference"
# beside this repository
REF="${NR_REFERENCE_DIR:-$(dirname "$(dirname "$HERE")")/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/Tomo_OSTR.cu" ] || [ ! -f "$REF/Tomo_OSTR_gold.cpp" ]; then
    echo "build_ref: reference sources not found under $REF" >&2
    exit 3
fi
mkdir -p "$OUT"
{
    echo '#include "ref_shim.h"'
    sed -n '18,116p;118,325p;327,610p;612,1173p;1177,1311p;1313,1449p;1453,1515p;1553,1735p;1737,2183p' \
        "$REF/Tomo_OSTR.cu"
    cat "$HERE/ref/ref_launch.inc"
    sed -n '22,1528p' "$REF/Tomo_OSTR_gold.cpp"
    cat "$HERE/ref/ref_api.inc"
} | g++ -x c++ -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w \
        -I "$HERE/ref" -o "$OUT/libostr_ref.so" -
echo "built $OUT/libostr_ref.so"
