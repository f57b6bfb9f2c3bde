#!/usr/bin/env bash
# Test infrastructure only. Compiles the reference engine's hot-path
# translation units straight from the reference source tree (never copied
# into this repository) together with oracle/ref_shim.cc into
# oracle/_ref/libaleator_ref.so, the reference-backed oracle used to pin the C
# restatement and to generate tests/golden fixtures.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: /root/reference)
# Exits 0 without building when the reference tree is absent.
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "build_ref: reference tree $REF not present; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
SRC="$REF/src"
TUS=(
  core/geometry/lattice.cc
  core/geometry/supercell.cc
  core/math/counter_based_rng.cc
  core/neighbor/cell_list.cc
  core/neighbor/verlet_list.cc
  forcefield/pairwise/lennard_jones.cc
  forcefield/electrostatics/ewald.cc
  forcefield/electrostatics/ewald_incremental_state.cc
  engines/monte_carlo/framework_energy_grid.cc
  engines/monte_carlo/monte_carlo_engine.cc
  engines/monte_carlo/peng_robinson.cc
  io/cif_document.cc
  io/symmetry_operation.cc
  io/element_table.cc
  io/structure_io.cc
)
# -ffp-contract=off keeps the reference's IEEE operation sequence on every
# host (no fused multiply-add contraction), matching the C restatement.
CXXFLAGS=(-std=c++23 -O2 -fPIC -ffp-contract=off -I"$SRC")
pids=()
objs=()
for tu in "${TUS[@]}"; do
  obj="$OUT/obj/$(echo "$tu" | tr '/' '_' | sed 's/\.cc$/.o/')"
  objs+=("$obj")
  g++ "${CXXFLAGS[@]}" -c "$SRC/$tu" -o "$obj" &
  pids+=($!)
done
g++ "${CXXFLAGS[@]}" -c "$HERE/ref_shim.cc" -o "$OUT/obj/ref_shim.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libaleator_ref.so" "${objs[@]}" "$OUT/obj/ref_shim.o"
# where the tests find the reference's own data files (structure files)
(cd "$REF" && pwd) > "$OUT/source_root"
echo "build_ref: wrote $OUT/libaleator_ref.so"
