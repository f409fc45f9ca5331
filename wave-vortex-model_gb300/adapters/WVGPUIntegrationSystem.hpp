// Reference-side drop-in: the GB300 library behind the reference's own C++
// interfaces.  A maintainer adds this header and WVGPUIntegrationSystem.cpp to
// the reference's PortableRuntime build (they include the reference's headers
// and include/wvgpu.h, and link libwvgpu.so); nothing in the GPU library
// depends on them.
//
//  * WVGPUKernelAdapter: the operations of WVTransformConstantStratificationKernel
//    (CompiledKernel/include/WaveVortexKernel/WVTransformConstantStratificationKernel.hpp:47-110)
//    that WVConstantStratificationForcingEngine calls
//    (PortableRuntime/src/WVForcingEngine.cpp:647-726,773-799,897-905), forwarded
//    to the C ABI with the reference's views, status codes and messages.
//  * WVGPUIntegrationSystem: a runtime::WVIntegrationSystem
//    (PortableRuntime/include/WaveVortexRuntime/WVIntegrationContracts.hpp:33-45)
//    whose right-hand side (nonlinear advection, optionally adaptive damping)
//    runs on the GPU, so the reference's own integrators (WVFixedStepRK4,
//    WVAdaptiveRK23) step it unchanged.
#pragma once

#include "wvgpu.h"

#include "WaveVortexKernel/WVKernelTypes.hpp"
#include "WaveVortexRuntime/WVForcingSchedule.hpp"
#include "WaveVortexRuntime/WVIntegrationContracts.hpp"

#include <memory>
#include <vector>

namespace wvgpu_adapter {

class WVGPUKernelAdapter {
public:
    // precision: WV_PRECISION_FP64 (the plain drop-in), WV_PRECISION_FP32X2 or WV_PRECISION_MIXED
    static wavevortex::WVKernelStatus create(const wavevortex::WVTransformConstantStratificationConfiguration& c,
                                             int precision, std::unique_ptr<WVGPUKernelAdapter>& out);
    ~WVGPUKernelAdapter();
    WVGPUKernelAdapter(const WVGPUKernelAdapter&) = delete;
    WVGPUKernelAdapter& operator=(const WVGPUKernelAdapter&) = delete;

    wavevortex::WVShape2D spectralShape() const noexcept { return shape_; }
    wavevortex::WVKernelStatus nonlinearFlux(const wavevortex::WVState& s, wavevortex::WVFlux& f);
    wavevortex::WVKernelStatus nonlinearFluxWithAdvectionFields(const wavevortex::WVState& s, wavevortex::WVFlux& f,
                                                                wavevortex::WVRealFieldBundleView& advection);
    wavevortex::WVKernelStatus nonlinearFluxUsingAdvectionFields(const wavevortex::WVState& s, wavevortex::WVFlux& f,
                                                                 const wavevortex::WVRealFieldBundleConstView& advection);
    wavevortex::WVKernelStatus transformWaveVortexToUVWEta(const wavevortex::WVState& s,
                                                           wavevortex::WVRealFieldBundleView& out);
    wavevortex::WVKernelStatus transformWaveVortexToUVW(const wavevortex::WVState& s, wavevortex::WVRealFieldBundleView& out);
    wavevortex::WVKernelStatus transformUVWEtaToWaveVortex(const wavevortex::WVRealFieldBundleConstView& in, double t,
                                                           double t0, wavevortex::WVMutableCoefficients& c);
    wavevortex::WVKernelStatus advectFGridScalar(const wavevortex::WVRealVolumeConstView& scalar,
                                                 const wavevortex::WVRealFieldBundleConstView& advection,
                                                 bool antialias, wavevortex::WVRealVolumeView& rhs);
    // The forcing schedule's right-hand side (WVIntegrationSystem::evaluateRightHandSide of
    // the coefficient-only system) and n WVFixedStepRK4 steps taken wholly on the GPU.
    wavevortex::WVKernelStatus setForcing(bool nonlinearAdvection, bool adaptiveDamping);
    wavevortex::WVKernelStatus evaluateRightHandSide(const wavevortex::WVState& s, wavevortex::WVFlux& f);
    wavevortex::WVKernelStatus rk4Steps(wavevortex::WVMutableState& s, double dt, int steps);
    wavevortex::WVKernelStatus errorTolerances(double scale, std::vector<double>& wave, std::vector<double>& vortex);
    wv_handle* handle() const noexcept { return h_; }

private:
    explicit WVGPUKernelAdapter(wv_handle* h, wavevortex::WVShape2D shape) : h_(h), shape_(shape) {}
    wavevortex::WVKernelStatus status(int rc) const;
    wv_handle* h_;
    wavevortex::WVShape2D shape_;
};

class WVGPUIntegrationSystem final : public wavevortex::runtime::WVIntegrationSystem {
public:
    // The schedule may hold WVNonlinearAdvection (required) and WVAdaptiveDamping,
    // as the compiled backend allows (WVTransformConstantStratification.m:616-621).
    static wavevortex::WVKernelStatus create(const wavevortex::WVTransformConstantStratificationConfiguration& c,
                                             const wavevortex::runtime::WVFrozenForcingSchedule& schedule, int precision,
                                             std::unique_ptr<WVGPUIntegrationSystem>& out);

    const wavevortex::runtime::WVIntegrationStateLayout& stateLayout() const noexcept override { return layout_; }
    wavevortex::WVKernelStatus evaluateRightHandSide(const wavevortex::runtime::WVIntegrationState& state,
                                                     wavevortex::runtime::WVIntegrationFlux& rightHandSide) override;
    wavevortex::runtime::WVStateConstraintResult enforceStateConstraints(
        wavevortex::runtime::WVMutableIntegrationState& state) override;
    wavevortex::WVKernelStatus createErrorPolicy(
        double absoluteToleranceScale, std::unique_ptr<wavevortex::runtime::WVIntegrationErrorPolicy>& policy) const override;

    WVGPUKernelAdapter& kernel() noexcept { return *kernel_; }
    std::size_t rightHandSideEvaluations() const noexcept { return evaluations_; }

private:
    WVGPUIntegrationSystem() = default;
    std::unique_ptr<WVGPUKernelAdapter> kernel_;
    wavevortex::runtime::WVIntegrationStateLayout layout_;
    std::size_t evaluations_ = 0;
};

} // namespace wvgpu_adapter
