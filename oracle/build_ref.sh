#!/usr/bin/env bash
# Test infrastructure: compiles the reference GRGL CPU matmul (and its constructor) from the
# sources where they lie under the reference checkout, into oracle/_ref/:
#   oracle/_ref/_grgl*.so     the reference Python module (pygrgl's `_grgl`), -O3 -DNDEBUG
#   oracle/_ref/ref_construct VCF/IGD -> .grg with the reference constructor
#   oracle/_ref/src           a link to the checkout (its test inputs and expected outputs)
#   oracle/_ref/pygrgl        a link to the checkout's Python package (which imports _grgl)
# Needs the reference checkout (GRGL_REF, default /root/reference) and pip pybind11.  Where the
# checkout is absent it does nothing and exits 0.  Nothing here is copied into the repository.
set -euo pipefail
REF=${GRGL_REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
if [ ! -f "$REF/include/grgl/grg.h" ]; then
  echo "reference checkout not found ($REF): oracle/_ref not built"
  exit 0
fi
python3 -c 'import pybind11' 2>/dev/null || { echo "pybind11 missing: oracle/_ref not built"; exit 0; }
OBJ=$OUT/obj
mkdir -p "$OBJ"
PYINC=$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
PBINC=$(python3 -c 'import pybind11; print(pybind11.get_include())')
EXT=$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
CXXFLAGS="-O3 -DNDEBUG -std=c++17 -fPIC -DVCF_GZ_SUPPORT=1 -I$HERE/ref_shim -I$REF/include -I$REF/src \
  -I$REF/third-party/libvbyte -I$REF/third-party/picovcf -I$REF/third-party/picohash -I$REF/third-party/hwe -w"
# libvbyte is compiled with -mavx on x86-64, as the reference build does (third-party/CMakeLists.txt:48-54).
VBFLAGS=""
[ "$(uname -m)" = "x86_64" ] && VBFLAGS="-mavx"
SRCS="grg serialize mutation transform map_mutations fast_build mut_iterator windowing grg_merge hap_index calculations"
pids=()
for s in $SRCS; do
  [ "$OBJ/$s.o" -nt "$REF/src/$s.cpp" ] 2>/dev/null || { g++ $CXXFLAGS -c "$REF/src/$s.cpp" -o "$OBJ/$s.o" & pids+=($!); }
done
g++ $CXXFLAGS -c "$REF/third-party/hwe/snp_hwe.cpp" -o "$OBJ/snp_hwe.o" & pids+=($!)
g++ $CXXFLAGS $VBFLAGS -c "$REF/third-party/libvbyte/vbyte.cc" -o "$OBJ/vbyte.o" & pids+=($!)
gcc -O3 -fPIC -w $VBFLAGS -c "$REF/third-party/libvbyte/varintdecode.c" -o "$OBJ/varintdecode.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref_shim/tsk_stubs.cpp" -o "$OBJ/tsk_stubs.o" & pids+=($!)
g++ $CXXFLAGS -I"$PYINC" -I"$PBINC" -c "$REF/src/python/_grgl.cpp" -o "$OBJ/_grgl.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref_construct.cpp" -o "$OBJ/ref_construct.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
CORE=""
for s in $SRCS; do CORE="$CORE $OBJ/$s.o"; done
CORE="$CORE $OBJ/snp_hwe.o $OBJ/vbyte.o $OBJ/varintdecode.o $OBJ/tsk_stubs.o"
g++ -shared -o "$OUT/_grgl$EXT" "$OBJ/_grgl.o" $CORE -lz -lpthread
g++ -o "$OUT/ref_construct" "$OBJ/ref_construct.o" $CORE -lz -lpthread
ln -sfn "$REF" "$OUT/src"
ln -sfn "$REF/pygrgl" "$OUT/pygrgl"
echo "built $OUT/_grgl$EXT and $OUT/ref_construct"
