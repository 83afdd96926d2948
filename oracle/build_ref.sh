#!/usr/bin/env bash
# Test infrastructure: builds the unmodified LASSIE reference binary into
# oracle/_ref/ (git-ignored).  Two steps, because the GPU machine is aarch64
# and has no copy of the reference project:
#   stage  (where the reference project is present): copy its four engine
#          sources into oracle/_ref/src/ unchanged -- never into tracked files;
#   build  (anywhere nvcc is): compile the staged sources with the
#          force-included oracle/ref_prelude.h into oracle/_ref/lassie_ref
#          (stock output) and oracle/_ref/lassie_ref_f64 (17-digit Solution).
# Usage: LASSIE_REFERENCE_DIR=<LASSIE checkout> oracle/build_ref.sh [stage|build|all]
#        (default: all; stage needs LASSIE_REFERENCE_DIR)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${LASSIE_REFERENCE_DIR:-}"
OUT="$HERE/_ref"
what="${1:-all}"
if [[ "$what" == stage || "$what" == all ]]; then
  if [[ -n "$REF" && -d "$REF/src/c++" ]]; then
    mkdir -p "$OUT/src/header"
    install -m 644 "$REF/src/c++/simulator.cu" "$OUT/src/"
    install -m 644 "$REF/src/c++/header/Simulation.cuh" "$REF/src/c++/header/kernels.cuh" \
       "$REF/src/c++/header/Reader.h" "$OUT/src/header/"
  fi
fi
if [[ "$what" == build || "$what" == all ]]; then
  if [[ ! -f "$OUT/src/simulator.cu" ]]; then
    echo "build_ref: no staged reference sources in $OUT/src" >&2
    exit 3
  fi
  flags=(-O3 --use_fast_math -restrict -gencode arch=compute_103a,code=sm_103a
         -include "$HERE/ref_prelude.h" -lcusolver -lcublas -w)
  nvcc "${flags[@]}" "$OUT/src/simulator.cu" -o "$OUT/lassie_ref" &
  p1=$!
  nvcc "${flags[@]}" -DLASSIE_REF_FULL_DIGITS "$OUT/src/simulator.cu" -o "$OUT/lassie_ref_f64" &
  p2=$!
  wait $p1
  wait $p2
fi
