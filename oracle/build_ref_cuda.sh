#!/bin/sh
# Builds oracle/_ref/<program>.cubin: the device code of the reference's own CUDA
# programs on the hot path, compiled unmodified from the reference tree for
# sm_103a.  Host code is not built (only cubins); oracle/ref_cuda.py loads them
# through the CUDA driver API and launches the reference kernels on device
# buffers.  The reference's helper_cuda.h reads cudaDeviceProp fields that CUDA
# 13 removed, so its include guard is predefined and oracle/ref_cuda_compat.h is
# force-included instead.  TEST INFRASTRUCTURE ONLY; needs the reference tree
# (default /root/reference).
set -e
REF=${SPACETIME_REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/Spin1GpeBCC/Spin1GpeBCC.cu" ] || { echo "reference tree not found at $REF" >&2; exit 3; }
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
build() {  # $1 = program path without .cu, $2 = output name
    d=$(dirname "$1")
    $NVCC -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -DHELPER_CUDA_H -w \
        -I"$REF" -I"$REF/$d" -include "$HERE/ref_cuda_compat.h" -o "$OUT/$2.cubin" "$REF/$1.cu"
}
build Spin1GpeBCC/Spin1GpeBCC spin1_bcc &
build Spin2GpeBCC/Spin2GpeBCC spin2_bcc &
build RelativisticSpin2Gpe/RelativisticSpin2Gpe rel_spin2_bcc &
build RelativisticSpin1Gpe/RelativisticSpin1Gpe rel_spin1_bcc &
build RelativisticGpeBCC/RelativisticGpeBCC rel_scalar_bcc &
build GrossPitaevskiiGpuBcc/GPUGrossPitaevskii_BCC scalar_bcc &
build GrossPitaevskiiGpuC15/GPUGrossPitaevskii_C15 scalar_c15 &
build GrossPitaevskiiGpuA15/GPUGrossPitaevskii_A15 scalar_a15 &
build GrossPitaevskiiGpuFcc/GPUGrossPitaevskii_FCC scalar_fcc &
wait
ls "$OUT"/*.cubin
