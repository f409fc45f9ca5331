// FP64 descriptor construction.  See wv_descriptor.hpp.  This translation unit
// is compiled with -ffp-contract=off: the mode order depends on Kh computed
// exactly as sqrt(k*k + l*l) without fused multiply-add.
#include "wv_descriptor.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>

namespace wvgpu {
namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;
// The F/G modal normalization uses 9.81 regardless of the configured g
// (WVKernelTypes.cpp:13-16).
constexpr double kModalNormalizationGravity = 9.81;

bool finite_positive(double v) { return std::isfinite(v) && v > 0.0; }

std::vector<int64_t> dft_modes(size_t n) {
    std::vector<int64_t> modes;
    const size_t positive = (n + 1) / 2;
    for (size_t v = 0; v < positive; ++v) modes.push_back(static_cast<int64_t>(v));
    for (size_t v = n / 2; v > 0; --v) modes.push_back(-static_cast<int64_t>(v));
    return modes;
}

size_t dft_index(int64_t mode, size_t n) { return mode >= 0 ? static_cast<size_t>(mode) : static_cast<size_t>(static_cast<int64_t>(n) + mode); }

}  // namespace

Status validate_config(const wv_config& c) {
    if (c.contract_version != WV_CONTRACT_VERSION) return {WV_INVALID_CONFIGURATION, "Unsupported kernel contract version."};
    if (c.Nx < 2 || c.Ny < 2 || c.Nz < 3 || c.Nj < 1 || c.Nj > c.Nz - 1)
        return {WV_INVALID_CONFIGURATION, "Nx and Ny must be at least 2, Nz at least 3, and Nj must lie in [1,Nz-1]."};
    if (!finite_positive(c.Lx) || !finite_positive(c.Ly) || !finite_positive(c.Lz) || !finite_positive(c.N0) ||
        !finite_positive(c.rho0) || !finite_positive(c.g) || !finite_positive(c.planetary_radius) ||
        !finite_positive(c.rotation_rate) || !std::isfinite(c.latitude) || std::abs(c.latitude) > 90.0)
        return {WV_INVALID_CONFIGURATION, "Physical lengths and constants must be finite and positive, and latitude must lie in [-90,90]."};
    const uint64_t lim = std::numeric_limits<uint64_t>::max();
    if (c.Nx > lim / c.Ny || c.Nx * c.Ny > lim / c.Nz) return {WV_SIZE_OVERFLOW, "shape element count overflow"};
    return {};
}

Status build_descriptor(const wv_config& c, Descriptor& d) {
    Status st = validate_config(c);
    if (!st) return st;
    d = Descriptor{};
    d.c = c;
    const size_t Nx = c.Nx, Ny = c.Ny, Nz = c.Nz, Nj = c.Nj;
    const auto kModes = dft_modes(Nx);
    const auto lModes = dft_modes(Ny);
    const double maxAbsK = 2.0 * kPi * (static_cast<double>(Nx / 2) / c.Lx);

    struct Mode { int64_t km, lm; double k, l, Kh; };
    std::vector<Mode> modes;
    for (const int64_t lm : lModes) {
        for (const int64_t km : kModes) {
            const bool kSelf = km == 0 || (Nx % 2 == 0 && km == -static_cast<int64_t>(Nx / 2));
            const bool lSelf = lm == 0 || (Ny % 2 == 0 && lm == -static_cast<int64_t>(Ny / 2));
            const bool primary = lm > 0 || (lSelf && (km > 0 || kSelf));
            const bool nyquist = (Nx % 2 == 0 && km == -static_cast<int64_t>(Nx / 2)) ||
                                 (Ny % 2 == 0 && lm == -static_cast<int64_t>(Ny / 2));
            if (!primary || nyquist) continue;
            const double k = 2.0 * kPi * (static_cast<double>(km) / c.Lx);
            const double l = 2.0 * kPi * (static_cast<double>(lm) / c.Ly);
            const double Kh = std::sqrt(k * k + l * l);
            if (c.should_antialias && Kh > 2.0 * maxAbsK / 3.0) continue;
            modes.push_back({km, lm, k, l, Kh});
        }
    }
    std::stable_sort(modes.begin(), modes.end(), [](const Mode& a, const Mode& b) {
        if (a.Kh != b.Kh) return a.Kh < b.Kh;
        if (a.km != b.km) return a.km < b.km;
        return a.lm < b.lm;
    });
    const size_t Nkl = modes.size();
    d.Nkl = Nkl;
    d.M = Nkl * Nj;
    d.NxHalf = Nx / 2 + 1;
    for (const auto& mo : modes) {
        d.kMode.push_back(mo.km);
        d.lMode.push_back(mo.lm);
        d.k.push_back(mo.k);
        d.l.push_back(mo.l);
        d.Kh.push_back(mo.Kh);
        d.cosAlpha.push_back(mo.Kh == 0.0 ? 0.0 : mo.k / mo.Kh);
        d.sinAlpha.push_back(mo.Kh == 0.0 ? 0.0 : mo.l / mo.Kh);
    }

    const double f = 2.0 * c.rotation_rate * std::sin(c.latitude * kPi / 180.0);
    d.f = f;
    d.z.resize(Nz);
    const double dz = c.Lz / static_cast<double>(Nz - 1);
    for (size_t i = 0; i < Nz; ++i) d.z[i] = dz * static_cast<double>(i) - c.Lz;
    d.m.resize(Nj); d.h0.resize(Nj); d.Fg.resize(Nj); d.Gg.resize(Nj); d.gWaveScale.resize(Nj);
    d.inertialScale.assign(Nj, 0.0); d.apmWProjectionPrefactor.assign(Nj, 0.0);
    for (size_t i = 0; i < Nj; ++i) {
        const double m = static_cast<double>(i) * kPi / c.Lz;
        d.m[i] = m;
        d.h0[i] = i == 0 ? c.Lz : c.N0 * c.N0 / (c.g * m * m);
    }
    const double N02 = c.N0 * c.N0;
    const double f2 = f * f;
    if (!c.is_hydrostatic && N02 <= f2)
        return {WV_INVALID_CONFIGURATION, "Nonhydrostatic constant stratification requires N0 squared greater than f squared."};
    for (size_t iJ = 0; iJ < Nj; ++iJ) {
        const double M = d.m[iJ];
        const double signNorm = iJ % 2 == 0 ? 1.0 : -1.0;
        const double Fg = iJ == 0 ? 2.0 : signNorm * d.h0[iJ] * M * std::sqrt(2.0 * kModalNormalizationGravity / (c.Lz * N02));
        const double Gg = iJ == 0 ? 1.0 : signNorm * std::sqrt(2.0 * kModalNormalizationGravity / (c.Lz * N02));
        const double Gw = c.is_hydrostatic || iJ == 0 ? Gg : signNorm * std::sqrt(2.0 * kModalNormalizationGravity / (c.Lz * (N02 - f2)));
        const double Gwg = Gg / Gw;
        d.Fg[iJ] = Fg;
        d.Gg[iJ] = Gg;
        d.gWaveScale[iJ] = Gg / Gwg;
    }

    const size_t M = d.M;
    auto zeros = [M](std::vector<double>& v) { v.assign(M, 0.0); };
    zeros(d.omega); zeros(d.fWaveScale); zeros(d.hpm); zeros(d.NAp); zeros(d.NA0); zeros(d.A0FromVorticity);
    zeros(d.A0FromBuoyancy); zeros(d.ApmN); zeros(d.ApmDScaled);
    for (auto* v : {&d.UAp, &d.VAp, &d.WAp, &d.UA0, &d.VA0, &d.ApmD}) v->assign(M, cdouble(0.0, 0.0));

    for (size_t iMode = 0; iMode < Nkl; ++iMode) {
        const double Kh = d.Kh[iMode];
        const double Kh2 = Kh * Kh;
        const double cosAlpha = d.cosAlpha[iMode];
        const double sinAlpha = d.sinAlpha[iMode];
        for (size_t iJ = 0; iJ < Nj; ++iJ) {
            const size_t index = iJ + Nj * iMode;
            const double Mv = d.m[iJ];
            const double signNorm = iJ % 2 == 0 ? 1.0 : -1.0;
            const bool isWave = Kh > 0.0 && iJ > 0;
            const bool isInertial = Kh == 0.0;
            const bool isGeostrophic = Kh > 0.0;
            const bool isMDA = Kh == 0.0 && iJ > 0;
            double hpm = 1.0;
            if (iJ > 0) hpm = c.is_hydrostatic ? N02 / (c.g * Mv * Mv) : (N02 - f2) / (c.g * (Mv * Mv + Kh2));
            const double Fg = d.Fg[iJ];
            const double Gg = d.Gg[iJ];
            double Fw = Fg;
            double Gw = Gg;
            if (!c.is_hydrostatic) {
                Fw = iJ == 0 ? 2.0 : signNorm * hpm * Mv * std::sqrt(2.0 * kModalNormalizationGravity / (c.Lz * (N02 - f2)));
                Gw = iJ == 0 ? 1.0 : signNorm * std::sqrt(2.0 * kModalNormalizationGravity / (c.Lz * (N02 - f2)));
            }
            const double omega = std::sqrt(c.g * hpm * Kh2 + f2);
            const double Fwg = Fg / Fw;
            const double Gwg = Gg / Gw;
            d.hpm[index] = hpm;
            d.omega[index] = omega;
            d.fWaveScale[index] = Fg / Fwg;
            if (iMode == 0) d.inertialScale[iJ] = 0.5 * Fwg / Fg;
            const double prefactor = signNorm * std::sqrt(c.g * c.Lz / (2.0 * (N02 - f2)));
            d.ApmDScaled[index] = (Mv / 2.0) * prefactor;
            if (iMode == 0) d.apmWProjectionPrefactor[iJ] = prefactor;
            if (isWave) {
                const double fs = d.fWaveScale[index];
                const double gs = d.gWaveScale[iJ];
                d.UAp[index] = cdouble(cosAlpha * fs, (-(f / omega) * sinAlpha) * fs);
                d.VAp[index] = cdouble(sinAlpha * fs, ((f / omega) * cosAlpha) * fs);
                d.WAp[index] = cdouble(0.0 * gs, (-Kh * hpm) * gs);
                d.NAp[index] = (-Kh * hpm / omega) * gs;
                const double deltaScale = d.h0[iJ] * Gwg / Fg;
                d.ApmD[index] = cdouble(0.0 * deltaScale, (-1.0 / (2.0 * Kh * hpm)) * deltaScale);
                d.ApmN[index] = (-omega / (2.0 * Kh * hpm)) * Gwg / Gg;
            } else if (isInertial) {
                d.UAp[index] = cdouble(d.fWaveScale[index], 0.0);
                d.VAp[index] = cdouble(0.0, d.fWaveScale[index]);
            }
            if (isGeostrophic) {
                const double Lr2Inverse = iJ == 0 ? 0.0 : f2 / (c.g * d.h0[iJ]);
                const double denominator = Kh2 + Lr2Inverse;
                d.UA0[index] = cdouble(0.0 * Fg, (d.l[iMode] / denominator) * Fg);
                d.VA0[index] = cdouble(0.0 * Fg, (-d.k[iMode] / denominator) * Fg);
                const double NA0 = iJ == 0 ? 0.0 : -(f / c.g) / denominator;
                d.NA0[index] = NA0 * Gg;
                d.A0FromVorticity[index] = 1.0 / Fg;
                d.A0FromBuoyancy[index] = iJ == 0 ? 0.0 : (-f / d.h0[iJ]) / Gg;
            } else if (isMDA) {
                d.NA0[index] = Gg;
                d.A0FromBuoyancy[index] = 1.0 / Gg;
                d.A0FromVorticity[index] = (f2 / (2.0 * d.h0[iJ])) / Fg;
            }
        }
    }

    const size_t NxHalf = d.NxHalf;
    const size_t halfRows = NxHalf * Ny;
    d.storageRow.resize(Nkl);
    d.conjugated.assign(Nkl, 0);
    std::vector<int64_t> represented(halfRows, -1);
    for (size_t i = 0; i < Nkl; ++i) {
        const int64_t km = d.kMode[i], lm = d.lMode[i];
        size_t row;
        if (km >= 0) {
            row = static_cast<size_t>(km) + NxHalf * dft_index(lm, Ny);
        } else {
            row = static_cast<size_t>(-km) + NxHalf * dft_index(-lm, Ny);
            d.conjugated[i] = 1;
        }
        d.storageRow[i] = row;
        represented[row] = static_cast<int64_t>(i);
    }
    std::vector<uint64_t> comp, src;
    for (size_t iL = 0; iL < Ny; ++iL) {
        const int64_t lm = iL <= Ny / 2 ? static_cast<int64_t>(iL) : static_cast<int64_t>(iL) - static_cast<int64_t>(Ny);
        const size_t destination = NxHalf * dft_index(lm, Ny);
        const size_t source = NxHalf * dft_index(-lm, Ny);
        if (represented[destination] < 0 && represented[source] >= 0) {
            comp.push_back(destination);
            src.push_back(source);
        }
        if (lm == 0 || (Ny % 2 == 0 && std::llabs(lm) == static_cast<int64_t>(Ny / 2))) {
            if (represented[destination] >= 0) d.selfConjugateRows.push_back(destination);
        }
    }
    d.completionRows.assign(comp.rbegin(), comp.rend());
    d.completionSources.assign(src.rbegin(), src.rend());
    return {};
}

namespace {
double vanishing_filter(double value, double cutoff, double maximum) {
    value = std::abs(value);
    if (value < cutoff) return 0.0;
    if (value > maximum) return 1.0;
    if (maximum == cutoff) return value >= maximum ? 1.0 : 0.0;
    const double ratio = (value - maximum) / (value - cutoff);
    return std::exp(-(ratio * ratio));
}
}  // namespace

Status adaptive_damping_operator(const Descriptor& d, std::vector<double>& damping) {
    const auto& c = d.c;
    const double f2 = d.f * d.f;
    if (!(f2 > 0.0)) return {WV_UNSUPPORTED_OPERATION, "Adaptive damping requires nonzero Coriolis frequency."};
    double maximumComponent = 0.0;
    for (size_t i = 0; i < d.Nkl; ++i) maximumComponent = std::max(maximumComponent, std::max(std::abs(d.k[i]), std::abs(d.l[i])));
    if (!(maximumComponent > 0.0)) return {WV_INVALID_CONFIGURATION, "Adaptive damping requires resolved horizontal wavenumbers."};
    const double effectiveResolution = kPi / maximumComponent;
    const double dklMinimum = std::min(2.0 * kPi / c.Lx, 2.0 * kPi / c.Ly);
    const double klCutoff = dklMinimum * std::pow(maximumComponent / dklMinimum, 0.75);
    const double jMaximum = static_cast<double>(c.Nj - 1);
    const double jCutoff = c.Nj > 2 ? std::pow(jMaximum, 0.75) : 0.0;
    const double prefactorXY = effectiveResolution / (kPi * kPi);
    const double referenceLr2 = c.g * d.h0.back() / f2;
    const double prefactorZ = (kPi * kPi * referenceLr2 / (effectiveResolution * effectiveResolution)) * prefactorXY;
    damping.assign(d.M, 0.0);
    for (size_t iMode = 0; iMode < d.Nkl; ++iMode) {
        const double Qkl = vanishing_filter(d.Kh[iMode], klCutoff, maximumComponent);
        for (size_t iJ = 0; iJ < c.Nj; ++iJ) {
            const size_t index = iJ + c.Nj * iMode;
            const double Qj = c.Nj > 2 ? vanishing_filter(static_cast<double>(iJ), jCutoff, jMaximum) : 1.0;
            const double Lr2Inverse = iJ == 0 ? 0.0 : f2 / (c.g * d.h0[iJ]);
            damping[index] = -prefactorXY * Qkl * d.Kh[iMode] * d.Kh[iMode] - prefactorZ * Qj * Lr2Inverse;
        }
    }
    return {};
}

Status adaptive_error_tolerances(const Descriptor& d, double absoluteScale, std::vector<double>& wave,
                                 std::vector<double>& vortex) {
    const auto& c = d.c;
    if (!std::isfinite(absoluteScale) || !(absoluteScale > 0.0))
        return {WV_INVALID_CONFIGURATION, "Adaptive absolute-tolerance scale must be finite and positive."};
    wave.assign(d.M, 1.0);
    vortex.assign(d.M, 1.0);
    // Radial shells of width dK (the widest gap between distinct |K_h|) centred
    // on 0, dK, 2 dK, ...; each coefficient of a shell gets an equal share of
    // the shell's width as its energy.
    std::vector<double> radii(d.Kh.begin(), d.Kh.end());
    for (double& r : radii) r = std::abs(r);
    std::sort(radii.begin(), radii.end());
    radii.erase(std::unique(radii.begin(), radii.end()), radii.end());
    if (radii.size() < 2)
        return {WV_INVALID_CONFIGURATION, "Adaptive tolerances require at least two distinct horizontal radial wavenumbers."};
    double dK = 0.0;
    for (size_t i = 1; i < radii.size(); ++i) dK = std::max(dK, radii[i] - radii[i - 1]);
    if (!(dK > 0.0) || !std::isfinite(dK)) return {WV_INVALID_CONFIGURATION, "Adaptive radial tolerance spacing is invalid."};
    std::vector<double> centres;
    for (double centre = 0.0; centre <= radii.back() + 0.5 * dK; centre += dK) centres.push_back(centre);
    std::vector<size_t> shell(d.Nkl, centres.size()), members(centres.size(), 0);
    for (size_t iMode = 0; iMode < d.Nkl; ++iMode) {
        for (size_t b = 0; b < centres.size(); ++b)
            if (centres[b] - 0.5 * dK < d.Kh[iMode] && d.Kh[iMode] <= centres[b] + 0.5 * dK) {
                shell[iMode] = b;
                ++members[b];
                break;
            }
        if (shell[iMode] == centres.size())
            return {WV_INVALID_CONFIGURATION, "A horizontal mode was not assigned to an adaptive radial tolerance bin."};
    }
    const double f2 = d.f * d.f, N02 = c.N0 * c.N0;
    for (size_t iMode = 0; iMode < d.Nkl; ++iMode) {
        const double Kh = d.Kh[iMode], Kh2 = Kh * Kh;
        const double centre = centres[shell[iMode]];
        const double width = centre + 0.5 * dK - std::max(centre - 0.5 * dK, 0.0);
        const double share = width / static_cast<double>(members[shell[iMode]]);
        for (size_t iJ = 0; iJ < c.Nj; ++iJ) {
            const size_t index = iJ + c.Nj * iMode;
            const double m = d.m[iJ];
            // energy per unit squared amplitude of the wave (A+/A-) and vortex (A0) parts
            double waveEnergy = 0.0;
            if (Kh == 0.0) {
                waveEnergy = iJ == 0 ? c.Lz : (c.is_hydrostatic ? N02 / (c.g * m * m) : (N02 - f2) / (c.g * m * m));
            } else if (iJ > 0) {
                waveEnergy = 2.0 * (c.is_hydrostatic ? N02 / (c.g * m * m) : (N02 - f2) / (c.g * (m * m + Kh2)));
            }
            double vortexEnergy = 0.0;
            if (Kh > 0.0) {
                const double Ld2Inverse = iJ == 0 ? 0.0 : f2 / (c.g * d.h0[iJ]);
                vortexEnergy = d.h0[iJ] / (Kh2 + Ld2Inverse);
            } else if (iJ > 0) {
                vortexEnergy = c.g / 2.0;
            }
            if (waveEnergy > 0.0 && std::isfinite(waveEnergy)) wave[index] = absoluteScale * std::sqrt(share / waveEnergy);
            if (vortexEnergy > 0.0 && std::isfinite(vortexEnergy)) vortex[index] = absoluteScale * std::sqrt(share / vortexEnergy);
        }
    }
    return {};
}

}  // namespace wvgpu
