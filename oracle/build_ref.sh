#!/usr/bin/env bash
# Builds oracle/_ref/libref_pd.so: the reference's own PD kernels
# (src/simulation/solver/projective/pdUtil.cu, with the templates of
# solverUtil.cuh and the vendored svd3_cuda/glm headers) compiled as C++
# through refshim/shim.h, plus refshim/ref_harness.cpp which drives them in
# the order PdSolver does.  Test infrastructure only; reads the reference
# sources where they lie and writes nothing outside oracle/_ref/.
#
# usage: build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
R="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=(g++ -std=c++17 -O2 -ffp-contract=off -fPIC -w)
INC=(-I"$HERE/refshim/include" -I"$R/src" -I"$R/src/simulation" -I"$R/src/simulation/solver"
     -I"$R/external/include" -I"$R/external/svd3_cuda")
"${CXX[@]}" -x c++ -include "$HERE/refshim/shim.h" "${INC[@]}" \
    -c "$R/src/simulation/solver/projective/pdUtil.cu" -o "$OUT/pdUtil.o"
"${CXX[@]}" -include "$HERE/refshim/shim.h" "${INC[@]}" -c "$HERE/refshim/ref_harness.cpp" -o "$OUT/ref_harness.o"
"${CXX[@]}" -fopenmp -c "$HERE/pd_oracle.cpp" -o "$OUT/pd_oracle.o"
g++ -shared -fopenmp -o "$OUT/libref_pd.so.tmp" "$OUT/pdUtil.o" "$OUT/ref_harness.o" "$OUT/pd_oracle.o"
mv "$OUT/libref_pd.so.tmp" "$OUT/libref_pd.so"
