#!/usr/bin/env bash
# Builds the reference's own CompiledKernel + PortableRuntime (fixed-RK4 subset) +
# direct-DFT reference FFT engine, straight from the reference checkout, into
# oracle/_ref/libwvref.so, together with oracle/ref_shim.cpp (a C entry layer).
# Test infrastructure only: used to generate golden fixtures and pin the oracle.
#
# Usage: oracle/ref_build.sh [REFERENCE_ROOT]   (default /root/reference)
# The file list and -DWV_MODEL_ENABLE_OUTPUT=0 follow the reference's own MEX
# build (@WVCompiledBackend/private/wvCompiledBackendBuild.m:272-309), with the
# FFTW engine replaced by adapters/reference/WVReferenceFFTEngine.cpp (FFTW is
# not installed here).
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/CompiledKernel" ]; then
  echo "reference checkout not found at $REF" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
CK="$REF/CompiledKernel"
PR="$REF/PortableRuntime"
SOURCES=(
  "$CK/src/WVKernelTypes.cpp"
  "$CK/src/WVTransformConstantStratificationKernel.cpp"
  "$CK/adapters/reference/WVReferenceFFTEngine.cpp"
  "$PR/src/WVExtensionCatalog.cpp"
  "$PR/src/WVPortableImplementationContract.cpp"
  "$PR/src/WVForcingContracts.cpp"
  "$PR/src/WVForcingEngine.cpp"
  "$PR/src/WVIntegrationState.cpp"
  "$PR/src/WVRungeKutta.cpp"
  "$PR/src/WVObserverAdapter.cpp"
  "$PR/src/WVObserverContracts.cpp"
  "$PR/src/WVObservation.cpp"
  "$PR/src/WVPortableTypedRecord.cpp"
  "$PR/src/WVOutputSchedule.cpp"
  "$PR/src/WVFieldEvaluationService.cpp"
  "$PR/src/WVConstantStratificationIntegrationSystem.cpp"
  "$PR/src/WVModel.cpp"
  "$HERE/ref_shim.cpp"
)
FLAGS=(-std=c++17 -O2 -fPIC -pthread -DWV_KERNEL_COEFFICIENT_WORKERS=2 -DWV_MODEL_ENABLE_OUTPUT=0
       -I"$CK/include" -I"$CK/src" -I"$CK/adapters/reference" -I"$PR/include" -I"$PR/src" -I"$PR/third_party")
pids=()
objs=()
for src in "${SOURCES[@]}"; do
  obj="$OUT/obj/$(basename "${src%.cpp}").o"
  objs+=("$obj")
  if [ ! -f "$obj" ] || [ "$src" -nt "$obj" ]; then
    g++ "${FLAGS[@]}" -c "$src" -o "$obj" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -pthread -o "$OUT/libwvref.so" "${objs[@]}"
echo "built $OUT/libwvref.so"
