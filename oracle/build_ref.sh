#!/usr/bin/env bash
# Builds oracle/_ref/libref_pd.so: the reference's own PD kernels
# (src/simulation/solver/projective/pdUtil.cu, with the templates of
# solverUtil.cuh and the vendored svd3_cuda/glm headers) compiled as C++
# through refshim/shim.h, plus refshim/ref_harness.cpp which drives them in
# the order PdSolver does, and the scene unit (fixed rigid bodies and the
# drag selection, see below).  Test infrastructure only; reads the reference
# sources where they lie and writes nothing outside oracle/_ref/.
#
# usage: build_ref.sh [REFERENCE_ROOT]
#   The reference root is the argument, else $PDGB_REFERENCE_ROOT, else the
#   place this container mounts it (/root/reference).  Where none of these
#   exists (the GPU machines) the script builds nothing and exits 0.  The root
#   used is recorded in oracle/_ref/REFERENCE_ROOT for the tests that read the
#   reference's own asset files.
set -euo pipefail
R="${1:-${PDGB_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$R/src/simulation/solver/projective" ]; then
    echo "build_ref.sh: no reference sources at $R; oracle/_ref not built" >&2
    exit 0
fi
mkdir -p "$OUT"
CXX=(g++ -std=c++17 -O2 -ffp-contract=off -fPIC -w)
INC=(-I"$HERE/refshim/include" -I"$R/src" -I"$R/src/simulation" -I"$R/src/simulation/solver"
     -I"$R/external/include" -I"$R/external/svd3_cuda")
"${CXX[@]}" -x c++ -include "$HERE/refshim/shim.h" "${INC[@]}" \
    -c "$R/src/simulation/solver/projective/pdUtil.cu" -o "$OUT/pdUtil.o"
"${CXX[@]}" -include "$HERE/refshim/shim.h" "${INC[@]}" -c "$HERE/refshim/ref_harness.cpp" -o "$OUT/ref_harness.o"
"${CXX[@]}" -fopenmp -c "$HERE/pd_oracle.cpp" -o "$OUT/pd_oracle.o"

# Scene unit: the reference's fixed-body kernels (fixedBodyData.cu), the
# constructors and getType of Plane / Sphere / Cylinder (collision/rigid/),
# FixedBody's constructors (rigid.cpp, compiled whole), the drag selection
# kernel Control_Kernel with its radius (simulationContext.cu) and
# utilityCore::modelMatrix (utilities.cpp).  Only the lines that hold them
# are read from those files and piped to the compiler -- the rest of each
# file launches kernels or draws with OpenGL -- so nothing is copied to disk.
RR="$R/src/collision/rigid"
SINC=("${INC[@]}" -I"$R/src/collision/rigid" -I"$HERE/refshim")
kernel_text() {  # kernel_text FILE NAME TEMPLATE-HEAD: one __global__ function, head line included
    awk -v name="$2" -v head="$3" '
        $0 ~ ("__global__ void " name "[ (]") { p = 1; print head }
        p { print }
        p && /^}/ { p = 0 }' "$1"
}
{
    echo '#include "fixed_prelude.h"'
    for k in Plane Sphere Cylinder; do
        f="$RR/$(echo "$k" | tr 'A-Z' 'a-z').cpp"
        sed -n "/^$k::$k(const glm::mat4/,/^{}/p" "$f"
        sed -n "/^BodyType $k::getType/,/^}/p" "$f"
    done
    for k in handleFloorCollision handleSphereCollision handleCylinderCollision; do
        kernel_text "$R/src/simulation/fixedBodyData.cu" "$k" 'template<typename Scalar>'
    done
    sed -n '/^#define RADIUS_SQUARED/p' "$R/src/simulation/simulationContext.cu"
    kernel_text "$R/src/simulation/simulationContext.cu" Control_Kernel 'template<class Scalar>'
    sed -n '/^glm::mat4 utilityCore::modelMatrix/,/^}/p' "$R/src/utilities.cpp"
    echo '#include "fixed_harness.inc"'
} | "${CXX[@]}" -x c++ -include "$HERE/refshim/shim.h" "${SINC[@]}" -c - -o "$OUT/ref_scene.o"
"${CXX[@]}" -include "$HERE/refshim/shim.h" "${SINC[@]}" -c "$RR/rigid.cpp" -o "$OUT/rigid.o"

# Collision unit: the reference's continuous-collision query from
# src/collision/intersections.cu -- stp, solveQuadratic, newtonsMethod,
# solveCubic, signed_vf_distance, signed_ee_distance and ccdCollisionTest --
# read function by function and piped to the compiler like the scene unit.
fn_text() {  # fn_text FILE NAME: one template function definition, its template line included
    awk -v name="$2" '
        /^template<typename (T|Scalar)>[ ]*$/ { hold = $0; next }
        {
            if (!p && hold != "" && index($0, " " name "(") > 0 && $0 !~ /\);[ ]*$/) {
                print hold; print; hold = ""
                if ($0 ~ /{/ && $0 ~ /}[ ]*$/) next
                p = 1; next
            }
            if (p) { print; if ($0 ~ /^}/) p = 0; next }
            hold = ""
        }' "$1"
}
{
    echo '#include "ccd_prelude.h"'
    for f in stp solveQuadratic newtonsMethod solveCubic signed_vf_distance signed_ee_distance ccdCollisionTest; do
        fn_text "$R/src/collision/intersections.cu" "$f"
    done
    echo '#include "ccd_harness.inc"'
} | "${CXX[@]}" -x c++ -include "$HERE/refshim/shim.h" "${SINC[@]}" -c - -o "$OUT/ref_ccd.o"
g++ -shared -fopenmp -o "$OUT/libref_pd.so.tmp" "$OUT/pdUtil.o" "$OUT/ref_harness.o" "$OUT/pd_oracle.o" \
    "$OUT/ref_scene.o" "$OUT/rigid.o" "$OUT/ref_ccd.o"
mv "$OUT/libref_pd.so.tmp" "$OUT/libref_pd.so"
printf "%s\n" "$(cd "$R" && pwd)" > "$OUT/REFERENCE_ROOT"
