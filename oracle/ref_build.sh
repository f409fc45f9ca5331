#!/usr/bin/env bash
# Builds the reference's own CompiledKernel + PortableRuntime (fixed-RK4 subset)
# with two FFT providers -- the reference's exact direct-DFT engine and the
# oracle's O(N log N) engine (oracle/wv_fft_engine.cpp) -- together with
# oracle/ref_shim.cpp (a C entry layer) into oracle/_ref/libwvref.so.
# Test infrastructure only: golden fixtures, parity at full grids, and the timed
# CPU baseline.  The GPU library never links or loads it.
#
# Usage: oracle/ref_build.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $WV_REFERENCE_ROOT, else /root/reference.
# When the reference checkout is present, the files of the subset (sources and
# headers, unmodified) are first staged into oracle/_ref/src (git-ignored), and
# the library is always compiled from that staged copy.  A machine without the
# checkout (the GPU host) builds from a staged copy that travelled with the
# working tree; without either the script exits 2.
# The file list and -DWV_MODEL_ENABLE_OUTPUT=0 follow the reference's own MEX
# build (@WVCompiledBackend/private/wvCompiledBackendBuild.m:272-309), with the
# FFTW engine replaced (FFTW is not installed here); -O3 and
# WV_KERNEL_NATIVE_OPTIMIZATION as that build sets them, without -mcpu=native so
# that one recipe serves both hosts.
set -euo pipefail
REF="${1:-${WV_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
STAGE="$OUT/src"
RUNTIME_SOURCES=(WVExtensionCatalog WVPortableImplementationContract WVForcingContracts WVForcingEngine
                 WVIntegrationState WVRungeKutta WVObserverAdapter WVObserverContracts WVObservation
                 WVPortableTypedRecord WVOutputSchedule WVFieldEvaluationService
                 WVConstantStratificationIntegrationSystem WVModel)

if [ -d "$REF/CompiledKernel" ] && [ -d "$REF/PortableRuntime" ]; then
  mkdir -p "$STAGE"
  # headers and sources of the subset, copied as they are (cp -u: only newer files)
  for d in CompiledKernel/include CompiledKernel/src CompiledKernel/adapters/reference \
           PortableRuntime/include PortableRuntime/third_party; do
    mkdir -p "$STAGE/$d"
    cp -ru "$REF/$d/." "$STAGE/$d/"
  done
  mkdir -p "$STAGE/PortableRuntime/src"
  find "$REF/PortableRuntime/src" -maxdepth 1 \( -name '*.hpp' -o -name '*.h' \) -exec cp -u {} "$STAGE/PortableRuntime/src/" \;
  for f in "${RUNTIME_SOURCES[@]}"; do cp -u "$REF/PortableRuntime/src/$f.cpp" "$STAGE/PortableRuntime/src/"; done
elif [ ! -d "$STAGE/CompiledKernel" ]; then
  echo "reference checkout not found at $REF and no staged copy in $STAGE" >&2
  exit 2
fi

mkdir -p "$OUT/obj"
CK="$STAGE/CompiledKernel"
PR="$STAGE/PortableRuntime"
SOURCES=(
  "$CK/src/WVKernelTypes.cpp"
  "$CK/src/WVTransformConstantStratificationKernel.cpp"
  "$CK/adapters/reference/WVReferenceFFTEngine.cpp"
)
for f in "${RUNTIME_SOURCES[@]}"; do SOURCES+=("$PR/src/$f.cpp"); done
SOURCES+=("$HERE/wv_fft_engine.cpp" "$HERE/ref_shim.cpp")
FLAGS=(-std=c++17 -O3 -fPIC -pthread -DWV_KERNEL_NATIVE_OPTIMIZATION=1 -DWV_KERNEL_COEFFICIENT_WORKERS=2
       -DWV_MODEL_ENABLE_OUTPUT=0
       -I"$HERE" -I"$CK/include" -I"$CK/src" -I"$CK/adapters/reference" -I"$PR/include" -I"$PR/src" -I"$PR/third_party")
pids=()
objs=()
for src in "${SOURCES[@]}"; do
  obj="$OUT/obj/$(basename "${src%.cpp}").o"
  objs+=("$obj")
  if [ ! -f "$obj" ] || [ "$src" -nt "$obj" ] || [ "$HERE/wv_fft_engine.hpp" -nt "$obj" ]; then
    g++ "${FLAGS[@]}" -c "$src" -o "$obj" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -pthread -o "$OUT/libwvref.so.tmp" "${objs[@]}"
mv "$OUT/libwvref.so.tmp" "$OUT/libwvref.so"
echo "built $OUT/libwvref.so"
