#!/usr/bin/env bash
# Builds the reference's own CPU tensor library (PyTAT, the pybind11 module `TAT`) from its
# sources under the read-only reference checkout into oracle/_ref/, for use as a checker only
# (golden-vector generation and cross-checks of the numpy restatement in oracle/).
#
# The reference's own build system is not used: the 32 scalar x symmetry instantiations of
# PyTAT/dealing_tensor.cpp.in are produced with sed and compiled with g++ directly.
# BLAS/LAPACK comes from scipy's bundled OpenBLAS, whose Fortran symbols carry a `scipy_` prefix;
# -D aliases map TAT's extern "C" names onto them.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: $TNSP_REFERENCE_ROOT)
set -euo pipefail
REF=${1:-${TNSP_REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then echo "usage: $0 REFERENCE_ROOT (or set TNSP_REFERENCE_ROOT)" >&2; exit 2; fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
GEN="$OUT/gen"
mkdir -p "$GEN"
if [ ! -d "$REF/PyTAT" ]; then echo "reference sources not found at $REF" >&2; exit 1; fi
PYINC=$(python3 -c "import sysconfig;print(sysconfig.get_paths()['include'])")
PB11=$(python3 -c "import pybind11;print(pybind11.get_include())")
SUFFIX=$(python3 -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
OPENBLAS=$(python3 -c "import scipy,glob,os;print(sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__)+'.libs','libscipy_openblas*.so')))[0])")
ALIASES=""
for p in s d c z; do
  for f in gemm gesvd geqrf gelqf gesv gemm_batch; do ALIASES="$ALIASES -D${p}${f}_=scipy_${p}${f}_"; done
done
for f in orgqr orglq; do for p in s d; do ALIASES="$ALIASES -D${p}${f}_=scipy_${p}${f}_"; done; done
for f in ungqr unglq; do for p in c z; do ALIASES="$ALIASES -D${p}${f}_=scipy_${p}${f}_"; done; done
CXXFLAGS="-O2 -std=c++17 -fPIC -DNDEBUG -DTAT_BUILD_TYPE=\"Release\" -I$REF/TAT/include -I$REF/PyTAT -I$PYINC -I$PB11 $ALIASES"
SRCS=("$REF/PyTAT/PyTAT.cpp")
Sy=(No BoseZ2 BoseU1 FermiU1 FermiU1BoseZ2 FermiU1BoseU1 FermiZ2 FermiU1FermiU1)
Sh=(S D C Z)
Sc=("float" "double" "std::complex<float>" "std::complex<double>")
for sym in "${Sy[@]}"; do
  for i in 0 1 2 3; do
    f="$GEN/dealing_tensor_${sym}_${Sh[$i]}.cpp"
    sed -e "s/@FUNCTION_NAME@/dealing_Tensor_${sym}_${Sh[$i]}/" -e "s/@SCALAR_NAME@/${Sc[$i]}/" \
        -e "s/@SYMMETRY_NAME@/${sym}Symmetry/" "$REF/PyTAT/dealing_tensor.cpp.in" > "$f.tmp"
    if ! cmp -s "$f.tmp" "$f"; then mv "$f.tmp" "$f"; else rm "$f.tmp"; fi
    SRCS+=("$f")
  done
done
OBJS=()
pids=()
for s in "${SRCS[@]}"; do
  o="$GEN/$(basename "$s" .cpp).o"
  OBJS+=("$o")
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then
    g++ $CXXFLAGS -c "$s" -o "$o" &
    pids+=($!)
    if [ ${#pids[@]} -ge "$(nproc)" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/TAT$SUFFIX" "${OBJS[@]}" "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")"
echo "built $OUT/TAT$SUFFIX"
