#!/bin/sh
# Builds oracle/_ref/<program>.cubin: the device code of the reference's own CUDA
# programs on the hot path, compiled unmodified from the reference tree for
# sm_103a.  Host code is not built (only cubins); oracle/ref_cuda.py loads them
# through the CUDA driver API and launches the reference kernels on device
# buffers.  The reference's helper_cuda.h reads cudaDeviceProp fields that CUDA
# 13 removed, so its include guard is predefined and oracle/ref_cuda_compat.h is
# force-included instead.  TEST INFRASTRUCTURE ONLY; needs the reference tree
# (default /root/reference).
#
# rel_spin2_gs.cubin holds the spin-2 ground-state kernels (itp_q, get_Hpsi,
# itp_psi), which the program compiles only with COMPUTE_GROUND_STATE set to 1;
# the file defines it as 0 unconditionally, so a transient copy with that one line
# changed is compiled (into _ref/, deleted afterwards) with the program's own
# directory on the include path.
set -e
REF=${SPACETIME_REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
# without the reference tree there is nothing to build: say so and succeed
[ -f "$REF/Spin1GpeBCC/Spin1GpeBCC.cu" ] || { echo "reference tree not found at $REF: oracle/_ref not built" >&2; exit 0; }
mkdir -p "$OUT"
# where the reference tree was found, for the tests that compare with its headers
echo "$REF" > "$OUT/ref_root.txt"
NVCC=${NVCC:-nvcc}
build() {  # $1 = program path without .cu, $2 = output name
    d=$(dirname "$1")
    $NVCC -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -DHELPER_CUDA_H -w \
        -I"$REF" -I"$REF/$d" -include "$HERE/ref_cuda_compat.h" -o "$OUT/$2.cubin" "$REF/$1.cu"
}
build_gs() {  # $1 = program path without .cu, $2 = output name
    d=$(dirname "$1")
    tmp="$OUT/.$2.cu"
    sed 's/^#define COMPUTE_GROUND_STATE 0$/#define COMPUTE_GROUND_STATE 1/' "$REF/$1.cu" > "$tmp"
    [ "$(grep -c '^#define COMPUTE_GROUND_STATE 1$' "$tmp")" = 1 ] || { echo "switch not found in $1.cu" >&2; rm -f "$tmp"; exit 4; }
    $NVCC -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -DHELPER_CUDA_H -w \
        -I"$REF" -I"$REF/$d" -include "$HERE/ref_cuda_compat.h" -o "$OUT/$2.cubin" "$tmp"
    rc=$?
    rm -f "$tmp"
    return $rc
}
build Spin1GpeBCC/Spin1GpeBCC spin1_bcc &
build Spin2GpeBCC/Spin2GpeBCC spin2_bcc &
build RelativisticSpin2Gpe/RelativisticSpin2Gpe rel_spin2_bcc &
build_gs RelativisticSpin2Gpe/RelativisticSpin2Gpe rel_spin2_gs &
build RelativisticSpin1Gpe/RelativisticSpin1Gpe rel_spin1_bcc &
build RelativisticGpeBCC/RelativisticGpeBCC rel_scalar_bcc &
build RelativisticGpeC15/GPUGrossPitaevskii_C15 rel_scalar_c15 &
build GrossPitaevskiiGpuBcc/GPUGrossPitaevskii_BCC scalar_bcc &
build GrossPitaevskiiGpuC15/GPUGrossPitaevskii_C15 scalar_c15 &
build GrossPitaevskiiGpuA15/GPUGrossPitaevskii_A15 scalar_a15 &
build GrossPitaevskiiGpuFcc/GPUGrossPitaevskii_FCC scalar_fcc &
wait
ls "$OUT"/*.cubin
