#!/usr/bin/env bash
# Builds the reference's own CUDA kernels, unmodified, from the reference
# sources where they lie, into device images under oracle/_ref/ (git-ignored).
# Test infrastructure: the kernels are run by oracle/ref_cuda.py to pin the
# oracle and to time the reference's plain kernel on the same GPU.
#
# Only device code is needed, so each file is compiled with -cubin (and -ptx as
# a JIT fallback); the programs' main() and host I/O are not built.  Flags as
# the reference would be built for this GPU: nvcc -O3 -arch=sm_103a.
# vissGen1M_shade_accurate.cu does not compile (`totalnode` undefined at :300)
# and is skipped.
set -euo pipefail
REF="${1:-/root/reference}"
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
[ -d "$REF" ] || { echo "reference sources not present: $REF" >&2; exit 0; }
mkdir -p "$OUT"
FILES="vissGen10M_shade vissGen10M_shade_optim1 vissGen10M_shade_optim2 vissGen1M_shade_optim1 \
vissGen1M_shade_optim2 vissGen1M_shade_appro MIncline_generate_uvw_float shade1M"
pids=()
for f in $FILES; do
  (
    if [ ! -f "$OUT/$f.cubin" ] || [ "$REF/$f.cu" -nt "$OUT/$f.cubin" ]; then
      nvcc -std=c++17 -O3 -arch=sm_103a -cubin -o "$OUT/$f.cubin" "$REF/$f.cu"
      nvcc -std=c++17 -O3 -arch=sm_103a -ptx -o "$OUT/$f.ptx" "$REF/$f.cu"
    fi
  ) &
  pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
