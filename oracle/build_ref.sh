#!/usr/bin/env bash
# Build the unmodified reference TwoChNRG NRG_main (and the reference-linked
# golden-vector harness) from the read-only reference tree, for use as a test
# oracle only.  Outputs go to oracle/_ref/ (git-ignored).  Needs the reference
# tree (REF_DIR; unset, the directory "reference" beside the repository) and scipy's bundled
# OpenBLAS for LAPACK/BLAS.  Nothing here is part of the product path.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
OBJ="$OUT/obj"
mkdir -p "$OBJ"
[ -d "$REF_DIR/src" ] || { echo "reference tree not found at $REF_DIR" >&2; exit 3; }

OPENBLAS="$(python3 - <<'PY'
import glob, os, scipy
d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
print(libs[0] if libs else "")
PY
)"
[ -n "$OPENBLAS" ] || { echo "scipy OpenBLAS not found" >&2; exit 3; }

CXX="${CXX:-g++}"
CXXFLAGS="-O2 -std=gnu++17 -fpermissive -w -I$HERE/ref_shim -I$REF_DIR/include -I$REF_DIR/src"

# The reference's NRG_main object list (src/Main/Makefile:16-28).
SRCS="NRGarrayClass NRGmatrixClass NRGthermoClass NRGchainClass ij2r r2ij CutStates
QS_BuildBasis CGordan_SStot CGordan dEqual CalcThermo Sdots QfdQm1 OpTables UpdateMatrices
FindMatchBlock CalcOpAvg FileExists DiagHN BuildBasis NRGcodehandlerClass OpMatRules
Calc_phMatEl TwoChQS_SetSingleSite TwoChQS_OpTables TwoChQS_OpMatRules CalcDN
CodeHandler_ModelSwitch HybFuncDefs SpecFuncClass GSL_Integrator SpecFunc_CFSmethod
SpecFunc_allSTL RotateMatrix"
MAIN_SRCS="Main_SetH0 Main_OpMatRules Main_SetSingleSite"

pids=()
compile() {  # $1 = source path, $2 = object path
  if [ ! -f "$2" ] || [ "$1" -nt "$2" ]; then "$CXX" $CXXFLAGS -c "$1" -o "$2"; fi
}
for s in $SRCS; do compile "$REF_DIR/src/$s.cpp" "$OBJ/$s.o" & pids+=($!); done
for s in $MAIN_SRCS; do compile "$REF_DIR/src/Main/$s.cpp" "$OBJ/$s.o" & pids+=($!); done
# OneChQS_SetSingleSite.cpp ends without a return statement (line 44), which
# GCC 13 compiles to a trap; compile it with the missing return supplied.
sed 's/^  \/\/ Important: SingleSite has Q,S,Sz block structure, one state per block/  return 0;/' \
  "$REF_DIR/src/OneChQS_SetSingleSite.cpp" > "$OBJ/OneChQS_SetSingleSite_ret.cpp"
compile "$OBJ/OneChQS_SetSingleSite_ret.cpp" "$OBJ/OneChQS_SetSingleSite.o" & pids+=($!)
gcc -O2 -c "$HERE/ref_shim/lapack_forward.c" -o "$OBJ/lapack_forward.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

LIBOBJS=""
for s in $SRCS $MAIN_SRCS OneChQS_SetSingleSite lapack_forward; do LIBOBJS="$LIBOBJS $OBJ/$s.o"; done
LDFLAGS="$OPENBLAS -Wl,-rpath,$(dirname "$OPENBLAS") -lm"

"$CXX" $CXXFLAGS "$REF_DIR/src/Main/NRG_main.cpp" $LIBOBJS $LDFLAGS -o "$OUT/NRG_main"
# DM_NRG (src/DM_NRG/Makefile: OBJS + OBJS_DMNRG) for the spectral-function
# golden vectors.
DM_SRCS="DM_NRG_SetChildSt DM_NRG_CalcRhoN DM_NRG_SetRhoNmax DM_NRG_CalcSpecFuncs DM_NRG_CommandLineRead"
pids=()
for s in $DM_SRCS; do compile "$REF_DIR/src/DM_NRG/$s.cpp" "$OBJ/$s.o" & pids+=($!); done
compile "$REF_DIR/src/BroadDelta.cpp" "$OBJ/BroadDelta.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
DMOBJS=""
for s in $DM_SRCS BroadDelta; do DMOBJS="$DMOBJS $OBJ/$s.o"; done
"$CXX" $CXXFLAGS "$REF_DIR/src/DM_NRG/DM_NRG.cpp" $DMOBJS $LIBOBJS $LDFLAGS -o "$OUT/DM_NRG"
if [ -f "$HERE/ref_harness.cpp" ]; then
  "$CXX" $CXXFLAGS "$HERE/ref_harness.cpp" $LIBOBJS $LDFLAGS -o "$OUT/ref_harness"
fi
echo "built $OUT/NRG_main"
