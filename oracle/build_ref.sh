#!/usr/bin/env bash
# TEST INFRASTRUCTURE.  Builds the reference demonstrator's own MFV code
# (jammartin/meshlessHydro) from its sources where they lie, with the shims in
# oracle/refshim/, into oracle/_ref/ (git-ignored).  Needs the reference tree
# (default /root/reference) and scipy's bundled OpenBLAS for dgetrf_/dgetri_;
# it runs only where both exist (not on the GPU host).
#
# Compiled reference files: demonstrator/src/{Particles,Domain,Helper,Riemann,
# Logger}.cpp.  Not compiled: main.cpp, ConfigParser.cpp (Boost, cxxopts),
# InitialDistribution.cpp (HDF5), MeshlessScheme.cpp (snapshots); the harness
# oracle/ref_harness.cpp drives the same stage sequence.
#
# Parameter sets: a forced-include header defines the reference's include
# guard DEMONSTRATOR_PARAMETER_H and the macros of demonstrator/include/
# parameter.h, so the in-tree parameter.h is skipped.  3D: demonstrator/
# include/Particles.h:43,54 declares z and vz only inside `#if RUNSPH`, and the
# SPH functions (Particles.cpp:367-1036) do not compile without periodic
# boundaries.  RUNSPH is therefore defined as (__COUNTER__ < 3): it is true for
# its first three uses in a translation unit (the declarations in Particles.h
# and the SPH allocations/deletions in the constructor and destructor,
# Particles.cpp:84,168) and false at Particles.cpp:367, so the MFV code builds
# unmodified and no SPH code is compiled or run.
#
# abs() binding: variants *_int see only <cmath>/<iostream>, where the
# unqualified abs(double) of Particles.cpp binds to int abs(int); variants
# *_dbl force-include <stdlib.h>, whose `using std::abs` makes it the double
# overload.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${MLH_REFERENCE:-/root/reference}"
# `build_ref.sh --print-root`: the reference tree this recipe reads (the one
# place that names its default location)
if [ "${1:-}" = "--print-root" ]; then echo "$REF"; exit 0; fi
SRC="$REF/demonstrator/src"
INC="$REF/demonstrator/include"
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -d "$SRC" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
BLAS="$(python3 - <<'PY'
import glob, os, scipy
d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
print(c[0] if c else "")
PY
)"
[ -n "$BLAS" ] || { echo "scipy OpenBLAS not found" >&2; exit 1; }

params() {  # name dim periodic cfl beta pairwise [first_order_quad_point 1] [finite_mass 0] [move 1] [slope 1]
  local f="$OUT/params_$1.h"
  cat > "$f" <<EOF
#ifndef DEMONSTRATOR_PARAMETER_H
#define DEMONSTRATOR_PARAMETER_H
#define DIM $2
#define PERIODIC_BOUNDARIES $3
#define ADAPTIVE_TIMESTEP 1
#define CFL $4
#define MAX_NUM_INTERACTIONS 400
#define MAX_NUM_GHOST_INTERACTIONS 300
#define SLOPE_LIMITING ${10:-1}
#define BETA $5
#define PAIRWISE_LIMITER $6
#define PSI_1 .5
#define PSI_2 .25
#define MESHLESS_FINITE_MASS ${8:-0}
#define ENFORCE_FLUX_SYM 1
#define MOVE_PARTICLES ${9:-1}
#define DEBUG_LVL 0
#define FIRST_ORDER_QUAD_POINT ${7:-1}
#define RUNSPH $([ "$2" = 3 ] && echo '(__COUNTER__ < 3)' || echo 0)
#define ARTVISC 0
#define VERBOSITY_PARTICLES 10
#define FLUX_SYM_TOL 1e-20
#endif
EOF
  echo "$f"
}

build() {  # variant params_header abs_mode
  local v="$1" ph="$2" absmode="$3"
  local extra=()
  [ "$absmode" = dbl ] && extra+=(-include stdlib.h)
  local objs=()
  for s in Particles Domain Helper Riemann Logger; do
    g++ -std=c++11 -O3 -ffp-contract=off -w -Dprivate=public -include "$ph" "${extra[@]}" \
        -I"$HERE/refshim" -I"$INC" -c "$SRC/$s.cpp" -o "$OUT/${v}_$s.o" &
    objs+=("$OUT/${v}_$s.o")
  done
  g++ -std=c++11 -O3 -ffp-contract=off -w -Dprivate=public -include "$ph" "${extra[@]}" \
      -I"$HERE/refshim" -I"$INC" -c "$HERE/ref_harness.cpp" -o "$OUT/${v}_harness.o" &
  gcc -O2 -c "$HERE/refshim/lapack_shim.c" -o "$OUT/${v}_lapack.o" &
  wait
  g++ -o "$OUT/ref_$v" "${objs[@]}" "$OUT/${v}_harness.o" "$OUT/${v}_lapack.o" \
      "$BLAS" -Wl,-rpath,"$(dirname "$BLAS")"
  echo "built $OUT/ref_$v"
}

KH=$(params kh 2 1 .3 4. 0)
KHPW=$(params khpw 2 1 .3 4. 1)
SED=$(params sedov 3 0 .25 1. 1)
SEDNP=$(params sedovnopw 3 0 .25 1. 0)
# the face point x_i + kernelSize/4 (x_j - x_i) instead of the midpoint; in 3D
# this path sets xjxi[2], so the 3D pairwise limiter is well defined there
KHQ=$(params khq 2 1 .3 4. 1 0)
SEDQ=$(params sedovq 3 0 .25 1. 1 0)
# the meshless finite mass scheme, and particles that do not move
KHMFM=$(params khmfm 2 1 .3 4. 0 1 1)
KHFIX=$(params khfix 2 1 .3 4. 0 1 0 0)
# no slope limiter
KHNOLIM=$(params khnolim 2 1 .3 4. 0 1 0 1 0)
build kh_dbl "$KH" dbl
build kh_int "$KH" int
build khpw_dbl "$KHPW" dbl
build khpw_int "$KHPW" int
build sedov_dbl "$SED" dbl
build sedov_int "$SED" int
build sedovnopw_dbl "$SEDNP" dbl
build khq_dbl "$KHQ" dbl
build sedovq_dbl "$SEDQ" dbl
build khmfm_dbl "$KHMFM" dbl
build khfix_dbl "$KHFIX" dbl
build khnolim_dbl "$KHNOLIM" dbl
