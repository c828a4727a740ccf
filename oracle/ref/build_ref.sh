#!/usr/bin/env bash
# Builds oracle/_ref/libahmed_ref.so: the reference library's hot-path sources
# compiled unmodified from the read-only reference tree, plus ref_driver.cpp.
# Runs only where the reference tree and scipy's bundled OpenBLAS exist; the
# output is test infrastructure (golden-vector generation), never shipped.
# The reference tree is AHMED_REF_DIR, by default the read-only copy of this
# build container.  --if-present: exit 0 quietly when the tree is absent (GPU
# hosts, which only use the committed fixtures).
set -euo pipefail
REF=${AHMED_REF_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/../_ref
if [ ! -d "$REF/Include" ]; then
  [ "${1:-}" = "--if-present" ] && exit 0
  echo "reference tree not found at $REF (set AHMED_REF_DIR)" >&2
  exit 2
fi
BLAS=$(python3 - <<'PY'
import glob, os, scipy
d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
print(c[0] if c else "")
PY
)
[ -n "$BLAS" ] || { echo "scipy OpenBLAS not found" >&2; exit 2; }
mkdir -p "$OUT/obj"
# Fortran BLAS/LAPACK names declared by the reference headers, mapped onto the
# scipy_-prefixed exports of the bundled OpenBLAS.
grep -ohE '\b[a-z][a-z0-9]*_\(' "$REF"/Include/*.h "$REF"/solvers/*.cpp | sed 's/($//' | sort -u > "$OUT/want.txt"
nm -D --defined-only "$BLAS" | awk '{print $3}' | grep '^scipy_' | sed 's/^scipy_//' | sort -u > "$OUT/have.txt"
ALIASES=$(comm -12 "$OUT/want.txt" "$OUT/have.txt" | sed 's/.*/-D&=scipy_&/' | tr '\n' ' ')
CXXFLAGS="-O2 -fopenmp -fPIC -DWIN32 -w -I$REF/Include $ALIASES"
# The whole non-MPI, non-METIS source set is compiled so that cross-file
# references (e.g. mltDiHGeM from H/mltaGeHVec.cpp) resolve without curation.
cd "$REF"
SRCS="$(ls H/*.cpp sparse/*.cpp solvers/*.cpp) cluster/AdjMatrix.cpp cluster/binSearch.cpp
      cluster/ClusterAlg.cpp cluster/specialSort.cpp cluster/CS_getPathAndDist.cpp
      cluster/blcluster.cpp parallel/gen_blseq.cpp basmod/progress.cpp"
cd "$HERE"
OBJS=""
printf '%s\n' $SRCS > "$OUT/srcs.txt"
export REF OUT CXXFLAGS
xargs -P "$(nproc)" -I{} sh -c 'g++ $CXXFLAGS -c "$REF/{}" -o "$OUT/obj/$(echo {} | tr / _).o"' < "$OUT/srcs.txt"
for s in $SRCS; do OBJS="$OBJS $OUT/obj/$(echo "$s" | tr '/' '_').o"; done
for c in basmod/realtime.c basmod/cputime.c; do
  gcc -O2 -fPIC -c "$REF/$c" -o "$OUT/obj/$(echo $c | tr / _).o"
  OBJS="$OBJS $OUT/obj/$(echo $c | tr / _).o"
done
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o"
g++ -shared -fopenmp -o "$OUT/libahmed_ref.so" $OBJS "$OUT/obj/ref_driver.o" \
    "$BLAS" -Wl,-rpath,"$(dirname "$BLAS")" -Wl,--no-undefined
echo "built $OUT/libahmed_ref.so"
