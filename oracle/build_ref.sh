#!/usr/bin/env bash
# Compile the reference's own HoughLine.cu device code (the vote kernels
# _houghlineImgKer / _houghlineCorKer and the drawing kernel _houghoutKer) and
# HoughCircle.cu device code (the vote kernel _houghcirImgKer) for sm_103a,
# straight from the reference tree, into oracle/_ref/.
# Only device code is produced: the fatbin is host-architecture neutral and is
# loaded on the GPU host by oracle/ref_runner.c through the driver API.
# Exit 3 when the reference tree is not mounted (e.g. on the GPU host, which
# then uses the fatbin built here).
set -euo pipefail
REF=/root/reference/okano_3_0
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/HoughLine.cu" ]; then
  exit 3
fi
mkdir -p "$OUT"
nvcc -fatbin -gencode arch=compute_103a,code=sm_103a -I"$REF" \
     "$REF/HoughLine.cu" -o "$OUT/houghline_ref.fatbin.tmp"
mv "$OUT/houghline_ref.fatbin.tmp" "$OUT/houghline_ref.fatbin"
nvcc -fatbin -gencode arch=compute_103a,code=sm_103a -I"$REF" \
     "$REF/HoughCircle.cu" -o "$OUT/houghcircle_ref.fatbin.tmp"
mv "$OUT/houghcircle_ref.fatbin.tmp" "$OUT/houghcircle_ref.fatbin"
