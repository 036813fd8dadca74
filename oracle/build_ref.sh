#!/usr/bin/env bash
# Builds the reference's own CUDA kernels, unmodified, from the reference
# sources where they lie, into device images under oracle/_ref/ (git-ignored).
# Test infrastructure: the kernels are run by oracle/ref_cuda.py to pin the
# oracle and to time the reference's kernels on the same GPU.
#
# Only device code is needed, so each file is compiled to a cubin for this GPU;
# the programs' main() and host I/O are not built.  Flags as the reference would
# be built for this GPU: nvcc -O3 -arch=sm_103a.
# vissGen1M_shade_accurate.cu does not compile (`totalnode` undefined at :300)
# and is skipped.
#
# Usage: build_ref.sh [reference-dir]; the directory defaults to
# $VISS_REFERENCE_DIR, else the reference checkout of the build container.
# Without the sources (the GPU machine) this is a no-op: the cubins built beside
# the sources travel with the repository copy.
set -euo pipefail
REF="${1:-${VISS_REFERENCE_DIR:-/root/reference}}"
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
[ -d "$REF" ] || { echo "reference sources not present: $REF" >&2; exit 0; }
mkdir -p "$OUT"
rm -f "$OUT"/*.ptx
FILES="vissGen10M_shade vissGen10M_shade_optim1 vissGen10M_shade_optim2 vissGen1M_shade_optim1 \
vissGen1M_shade_optim2 vissGen1M_shade_appro MIncline_generate_uvw_float shade1M"
pids=()
for f in $FILES; do
  (
    if [ ! -f "$OUT/$f.cubin" ] || [ "$REF/$f.cu" -nt "$OUT/$f.cubin" ]; then
      nvcc -std=c++17 -O3 -arch=sm_103a -cubin -o "$OUT/$f.cubin" "$REF/$f.cu"
    fi
  ) &
  pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
