#!/bin/sh
# Builds oracle/_ref/smaiso_wcomp_ref: the reference's own time loop
# (smaiso-wcomp.cpp), compiled from its source where it lies, against the
# MPI/FFTW-MPI stand-in in oracle/refshim/. TEST INFRASTRUCTURE ONLY: its outputs
# pin the oracle (tests/golden/make_ref_fixtures.py).
#
# The source is read, never copied: sed applies the substitutions below to the
# stream that g++ compiles. Each one changes what a run of the reference is sized
# or instrumented with, not what a step computes:
#   1. grid (:218)           Nx, Ny, Nz = 512 -> swc_ref_dim(0..2) (SWC_REF_NX/NY/NZ)
#   2. output root (:184,198) "/box/..." -> swc_ref_box() + "/..." (SWC_REF_DIR)
#   3. step count (:1081)    while (L1 > limL1) gains && nLoop < swc_ref_nsteps()
#   4. initial psi (:710)    after the reference's own IC, psi_local may be read
#                            from SWC_REF_PSI0 (swc_ref_initial_psi)
#   5. diagnostics (:2265)   after Bcast(&L1): SWC_REF_DIAG() records L1, the sums,
#                            mass and energy at full precision (the text files keep
#                            6 digits)
#   6. end of a step (:2457) SWC_REF_AFTER_STEP() writes the 24 fields at the steps
#                            listed in SWC_REF_DUMP
# and main is renamed swc_ref_main (-Dmain=...) so the stand-in's launcher can fork
# the ranks. dt, the coefficients and every stage are the reference's.
#
# usage: build_ref.sh <path of smaiso-wcomp.cpp> <output dir>
set -eu
SRC=$1
OUT=$2
HERE=$(cd "$(dirname "$0")" && pwd)
CXX=${CXX:-g++}
CC=${CC:-gcc}

if [ ! -r "$SRC" ]; then
  echo "build_ref.sh: reference source $SRC not found" >&2
  exit 2
fi
mkdir -p "$OUT"

patch_stream() {
  sed \
    -e 's/const ptrdiff_t Nx = 512, Ny = 512, Nz = 512;/const ptrdiff_t Nx = swc_ref_dim(0), Ny = swc_ref_dim(1), Nz = swc_ref_dim(2);/' \
    -e 's|std::string strLoad = "/box/|std::string strLoad = swc_ref_box() + "/|' \
    -e 's|std::string strBox = "/box/|std::string strBox = swc_ref_box() + "/|' \
    -e 's/while (L1 > limL1)$/while (L1 > limL1 \&\& nLoop < swc_ref_nsteps())/' \
    -e 's|^/\* Output IC to file  \*/$|swc_ref_initial_psi(psi_local.data(), local_n0, local_0_start);\n&|' \
    -e 's|MPI::COMM_WORLD.Bcast(&L1,1,MPI::DOUBLE,0);$|&\n      SWC_REF_DIAG();|' \
    -e 's|^} // End: time loop$|SWC_REF_AFTER_STEP();\n&|' \
    "$SRC"
}

# Every substitution must apply exactly once (a silent miss would, e.g., leave the
# grid at 512^3): 3 dims + 2 paths + 1 step limit + 1 IC hook + 2 probes.
N=$(patch_stream | grep -o 'swc_ref_dim(\|swc_ref_box()\|swc_ref_nsteps()\|swc_ref_initial_psi(\|SWC_REF_DIAG()\|SWC_REF_AFTER_STEP()' | wc -l)
if [ "$N" -ne 9 ]; then
  echo "build_ref.sh: expected 9 substituted hooks, found $N (reference source changed?)" >&2
  exit 3
fi

FLAGS="-O2 -ffp-contract=off -fopenmp"
$CC $FLAGS -std=c11 -c -o "$OUT/swc_oracle_r2r.o" "$HERE/swc_oracle.c"
$CXX $FLAGS -std=c++17 -c -o "$OUT/refshim.o" "$HERE/refshim/refshim.cpp"
patch_stream | $CXX $FLAGS -std=c++17 -w -D_GLIBCXX_ASSERTIONS -Dmain=swc_ref_main \
  -I"$HERE/refshim" -x c++ -c -o "$OUT/smaiso_wcomp.o" -
$CXX -fopenmp -o "$OUT/smaiso_wcomp_ref" "$OUT/smaiso_wcomp.o" "$OUT/refshim.o" \
  "$OUT/swc_oracle_r2r.o" -lm -lpthread
echo "built $OUT/smaiso_wcomp_ref"
