#!/usr/bin/env bash
# Builds the reference project's own code from its read-only sources into
# oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY: the outputs generate
# golden vectors under tests/golden/ and are never linked into the product.
#
#   oracle/_ref/intended/_core*.so   reference pybind module (core/bindings/pybind_module.cpp)
#                                    with the CPU core and GpuSolver driver
#                                    (core/src/gpu/gpu_solver.cpp) running the
#                                    reference kernels (core/src/gpu/cuda_pdhg.cu)
#                                    on the CPU; int64 index copies converted
#                                    to int32 (the intended gpu_solver.cpp:202-203)
#   oracle/_ref/faithful/_core*.so   same, with the shipped byte-for-byte copy
#   oracle/_ref/engine/_core*.so     the reference pybind module with gpu_solver.cpp
#                                    replaced by refinery-optimizer_gb300/host/
#                                    gpu_solver_adapter.cpp, linked to the engine's
#                                    libsih_pdhg.so (the drop-in, built when that
#                                    library exists)
#
# The CUDA runtime is replaced by oracle/ref_emul/cuda_runtime.h and the kernel
# launch syntax by oracle/ref_emul/ref_launchers.cpp.  Nothing else is
# changed; no reference file is copied into the repository.
# Usage: oracle/ref_build.sh [reference_dir]   (exits 0 when the reference is absent)
#        oracle/ref_build.sh --print-dir        prints the reference directory if its
#                                               sources are there (nothing otherwise)
# The reference directory is SIH_REFERENCE_DIR, else this recipe's default; the
# tests and the build entry point ask this recipe for it (oracle.reference_dir()).
set -euo pipefail
if [ "${1:-}" = "--print-dir" ]; then
    R="${SIH_REFERENCE_DIR:-/root/reference}"
    if [ -d "$R/core/src" ]; then echo "$R"; fi
    exit 0
fi
REF="${1:-${SIH_REFERENCE_DIR:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/core/src" ]; then
    echo "ref_build: reference sources not found at $REF; nothing built"
    exit 0
fi
mkdir -p "$OUT/obj" "$OUT/intended" "$OUT/faithful"
# kernel definitions only: stop before the launchers (which use <<<>>>) and drop
# the file-level #ifdef SIH_CUDA_ENABLED, whose #endif is in the part left out
awk '/Host Entry Functions/{exit} !/^#ifdef SIH_CUDA_ENABLED/{print}' "$REF/core/src/gpu/cuda_pdhg.cu" > "$OUT/ref_kernels.inc"

CXX="${CXX:-g++}"
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
PYBIND="$(python3 -c 'import pybind11; print(pybind11.get_include())')"
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
FLAGS="-std=c++17 -O2 -fPIC -fopenmp -ffp-contract=off -w -I$REF/core/include"

SRCS="model/sparse_matrix model/problem model/solution model/options io/mps_io checker/checker
telemetry/telemetry utils/affinity scaling/scaler factorization/sparse_lu factorization/amd
factorization/sparse_cholesky factorization/sparse_ldl presolve/presolver simplex/dual_simplex
simplex/primal_simplex simplex/simplex_solver ipm/crossover ipm/ipm_solver bnb/milp_presolve
bnb/gomory_cuts bnb/heuristics bnb/branch_and_bound"

for s in $SRCS; do
    o="$OUT/obj/$(basename "$s").o"
    [ "$o" -nt "$REF/core/src/$s.cpp" ] || $CXX $FLAGS -c "$REF/core/src/$s.cpp" -o "$o" &
done
wait
[ "$OUT/obj/pybind_module.o" -nt "$REF/core/bindings/pybind_module.cpp" ] || \
    $CXX $FLAGS -I"$PYINC" -I"$PYBIND" -c "$REF/core/bindings/pybind_module.cpp" -o "$OUT/obj/pybind_module.o"

for variant in intended faithful; do
    vflag=""
    [ "$variant" = intended ] && vflag="-DSIH_EMUL_INTENDED_INDEX_COPY"
    vo="$OUT/$variant"
    $CXX $FLAGS $vflag -DSIH_CUDA_ENABLED -I"$HERE/ref_emul" -c "$REF/core/src/gpu/gpu_solver.cpp" -o "$vo/gpu_solver.o" &
    $CXX $FLAGS $vflag -I"$HERE/ref_emul" -I"$OUT" -c "$HERE/ref_emul/ref_launchers.cpp" -o "$vo/ref_launchers.o" &
    wait
    $CXX -shared -fopenmp -o "$vo/_core$EXT" "$OUT"/obj/*.o "$vo/gpu_solver.o" "$vo/ref_launchers.o"
done
ENGINE_LIB="$HERE/../refinery-optimizer_gb300/_build"
if [ -f "$ENGINE_LIB/libsih_pdhg.so" ]; then
    mkdir -p "$OUT/engine"
    $CXX $FLAGS -I"$HERE/../include" -c "$HERE/../refinery-optimizer_gb300/host/gpu_solver_adapter.cpp" \
        -o "$OUT/engine/gpu_solver_adapter.o"
    $CXX -shared -fopenmp -o "$OUT/engine/_core$EXT" "$OUT"/obj/*.o "$OUT/engine/gpu_solver_adapter.o" \
        -L"$ENGINE_LIB" -lsih_pdhg -Wl,-rpath,"$ENGINE_LIB"
    echo "ref_build: built $OUT/engine/_core$EXT (reference bindings over the engine)"
fi
echo "ref_build: built $OUT/intended/_core$EXT and $OUT/faithful/_core$EXT"
