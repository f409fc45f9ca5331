// Host-side FP64 descriptor of the constant-stratification wave-vortex
// transform: WV mode set and canonical order, vertical modes, dispersion
// relation and every projection/reconstruction coefficient array, plus the
// half-spectrum mappings.  Built once per handle and uploaded to HBM.
//
// Follows WVTransformConstantStratificationDescriptor::create
// (CompiledKernel/src/WVKernelTypes.cpp:119-330).  Compiled without
// floating-point contraction so that Kh = sqrt(k*k + l*l) and every
// coefficient match the reference bit for bit (WVKernelTypes.cpp:22-29).
#pragma once

#include "wvgpu.h"

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

namespace wvgpu {

using cdouble = std::complex<double>;

struct Status {
    int code = WV_SUCCESS;
    std::string message;
    explicit operator bool() const { return code == WV_SUCCESS; }
};

struct Descriptor {
    wv_config c{};
    size_t Nkl = 0, M = 0, NxHalf = 0;
    double f = 0.0;
    // Horizontal modes in canonical WV order [Nkl].
    std::vector<int64_t> kMode, lMode;
    std::vector<double> k, l, Kh, cosAlpha, sinAlpha;
    // Vertical [Nj] / [Nz].
    std::vector<double> z, m, h0, Fg, Gg, gWaveScale, inertialScale, apmWProjectionPrefactor;
    // Coefficient arrays [Nj, Nkl] (j fastest).
    std::vector<double> omega, fWaveScale, hpm, NAp, NA0, A0FromVorticity, A0FromBuoyancy, ApmN, ApmDScaled;
    std::vector<cdouble> UAp, VAp, WAp, UA0, VA0, ApmD;
    // Half-spectrum mappings (WVKernelTypes.cpp:286-321).
    std::vector<uint64_t> storageRow;      // [Nkl]
    std::vector<uint8_t> conjugated;       // [Nkl]
    std::vector<uint64_t> completionRows, completionSources, selfConjugateRows;
};

Status validate_config(const wv_config& c);
Status build_descriptor(const wv_config& c, Descriptor& d);

// Adaptive-damping operator [Nj, Nkl] (PortableRuntime/src/WVForcingEngine.cpp:30-38,352-381).
Status adaptive_damping_operator(const Descriptor& d, std::vector<double>& damping);

// Absolute error tolerances of the adaptive RK23 controller, [Nj, Nkl] each:
// wave for A+ and A-, vortex for A0 (WVWaveVortexCoefficientErrorPolicy::create,
// PortableRuntime/src/WVForcingEngine.cpp:79-168).  Entries without a finite
// positive energy factor keep 1.
Status adaptive_error_tolerances(const Descriptor& d, double absoluteScale, std::vector<double>& wave,
                                 std::vector<double>& vortex);

}  // namespace wvgpu
