#!/usr/bin/env bash
# Compiles the reference's own CPU energy path (gpuATTRACT 2.0, unmodified
# sources read in place) together with oracle/ref_driver.cpp into
# oracle/_ref/libattract_ref.so.  Test infrastructure only: it pins the C++
# restatement in attract_oracle.cpp and writes the golden fixtures.
# Needs the reference tree (REF_ROOT, default /root/reference); exits 0 with a
# message when it is absent (the GPU machine has no copy of it).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF_ROOT/src/model" ]; then
	echo "build_ref: reference sources not found at $REF_ROOT; skipping"
	exit 0
fi
mkdir -p "$OUT/obj"
SRC="$REF_ROOT/src"
INC=""
for d in $(find "$SRC" -maxdepth 2 -type d); do INC="$INC -I$d"; done
FILES="model/Protein.cpp model/IntrplGrid.cpp model/NLGrid.cpp model/GridUnion.cpp
model/TypeMap.cpp model/Types_6D.cpp model/Types_6D_Modes.cpp model/DOFTransform.cpp
service/CPUEnergyService6D.cpp service/CPUEnergyService6DModes.cpp
server/DataManager.cpp server/Thread.cpp server/Server.cpp
fileIO/readFile.cpp fileIO/grid_orig.cpp"
# the reference's release flags (Makefile: -O3 -DNDEBUG -std=c++11), no CUDA;
# -ffp-contract=off keeps its float arithmetic unfused on every host
FLAGS="-O3 -DNDEBUG -std=c++11 -fPIC -ffp-contract=off -w"
pids=()
objs=()
for f in $FILES; do
	o="$OUT/obj/$(echo "$f" | tr '/' '_' | sed 's/\.cpp$/.o/')"
	objs+=("$o")
	if [ ! -f "$o" ] || [ "$SRC/$f" -nt "$o" ]; then
		g++ $FLAGS $INC -c "$SRC/$f" -o "$o" &
		pids+=($!)
	fi
done
g++ $FLAGS $INC -I"$HERE" -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libattract_ref.so" "${objs[@]}" "$OUT/obj/ref_driver.o" -lpthread
# tests locate the reference test resources through this marker
echo "$REF_ROOT" > "$OUT/ref_root.txt"
echo "build_ref: wrote $OUT/libattract_ref.so"
