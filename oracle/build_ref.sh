#!/usr/bin/env bash
# Builds oracle/_ref/ref_harness from the reference's own hot-path sources,
# unmodified, against the shim headers in oracle/ref_shim (Eigen, nlohmann_json,
# Boost and MPI are not installed here). Test infrastructure only: the binary
# generates the golden vectors under tests/golden/ and is never part of the
# product. Uses the reference's Release flags (CMakeLists.txt:56-58) except
# -ffp-contract=fast, replaced by -ffp-contract=off so x86-64 and aarch64 builds
# round identically.
#
# usage: oracle/build_ref.sh [reference_root]
#   reference_root defaults to $LMC_REFERENCE_ROOT, else /root/reference
set -euo pipefail
REF=${1:-${LMC_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/lmc" ]; then
  echo "reference sources not found at $REF; oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
R="$REF/lmc"
CXXFLAGS="-std=c++20 -O3 -fno-math-errno -fno-trapping-math -ffp-contract=off -fopenmp"
INC="-I$HERE/ref_shim -I$R/cfg/include -I$R/pred/include -I$R/mc/include -I$R/api/include"
SRCS="cfg/src/Config.cpp pred/src/EnergyUtility.cpp pred/src/VacancyMigrationPredictorQuartic.cpp
      pred/src/VacancyMigrationPredictorQuarticLru.cpp pred/src/VacancyMigrationPredictorE0.cpp
      pred/src/EnergyChangePredictorPairSite.cpp pred/src/EnergyPredictor.cpp
      pred/src/TimeTemperatureInterpolator.cpp mc/src/McAbstract.cpp mc/src/KineticMcAbstract.cpp
      mc/src/KineticMcFirstOmp.cpp mc/src/JumpEvent.cpp mc/src/CanonicalMcAbstract.cpp
      mc/src/CanonicalMcOmp.cpp mc/src/CanonicalMcSerial.cpp mc/src/ThermodynamicAveraging.cpp"
pids=()
OBJS=()
for f in $SRCS; do
  o="$OUT/obj/$(basename "$f" .cpp).o"
  OBJS+=("$o")
  g++ $CXXFLAGS $INC -c "$R/$f" -o "$o" &
  pids+=($!)
done
g++ $CXXFLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ $CXXFLAGS -o "$OUT/ref_harness" "$OUT/obj/ref_harness.o" "${OBJS[@]}" -lz
echo "built $OUT/ref_harness"
