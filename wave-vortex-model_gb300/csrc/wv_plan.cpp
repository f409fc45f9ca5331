// Layout plan construction (host).  See wv_plan.hpp.
#include "wv_plan.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace wvgpu {
namespace {
constexpr double kPi = 3.141592653589793238462643383279502884;

// cos(pi * a / b) and sin(pi * a / b) with the argument reduced exactly in
// integers first, so every matrix entry is correctly rounded to ~1 ulp.
double cospi_ratio(long long a, long long b) {
    long long r = a % (2 * b);
    if (r < 0) r += 2 * b;
    // pi*r/b in [0, 2pi)
    return std::cos(kPi * static_cast<double>(r) / static_cast<double>(b));
}
double sinpi_ratio(long long a, long long b) {
    long long r = a % (2 * b);
    if (r < 0) r += 2 * b;
    if (r == 0 || r == b) return 0.0;
    return std::sin(kPi * static_cast<double>(r) / static_cast<double>(b));
}

std::vector<double> twiddles(int N) {
    std::vector<double> t(2 * static_cast<size_t>(N));
    for (int k = 0; k < N; ++k) {
        // exp(-2 pi i k / N) = cos(pi*2k/N) - i sin(pi*2k/N)
        t[2 * k] = cospi_ratio(2LL * k, N);
        t[2 * k + 1] = -sinpi_ratio(2LL * k, N);
    }
    return t;
}
}  // namespace

FFTFactors factor_fft(int N) {
    FFTFactors f;
    f.N = N;
    int n = N;
    auto push = [&](int r) { if (f.nstages < kMaxStages) f.radix[f.nstages++] = r; };
    while (n % 4 == 0) { push(4); n /= 4; }
    while (n % 2 == 0) { push(2); n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) { push(p); n /= p; }
        if (p * p > n && n > 1) { push(n); n = 1; }
    }
    return f;
}

Status build_plan(const Descriptor& d, Plan& p) {
    const auto& c = d.c;
    p = Plan{};
    p.Nx = c.Nx; p.Ny = c.Ny; p.Nz = c.Nz; p.Nj = c.Nj; p.Nkl = d.Nkl; p.NxHalf = d.NxHalf; p.M = d.M;
    if (p.Nx > static_cast<size_t>(kMaxFFT) || p.Ny > static_cast<size_t>(kMaxFFT))
        return {WV_UNSUPPORTED_OPERATION, "Nx and Ny above 1024 are not supported by the GPU transforms."};
    if (c.is_hydrostatic) { p.targets.count = 3; p.targets.q[0] = 0; p.targets.q[1] = 1; p.targets.q[2] = 3; }
    else { p.targets.count = 4; for (int i = 0; i < 4; ++i) p.targets.q[i] = i; }

    // Active rows: retained storage rows and completion rows.
    struct Row { int64_t kx, ky; int32_t mode; int32_t compOf; };
    std::vector<Row> rows;
    const size_t NxHalf = p.NxHalf;
    for (size_t i = 0; i < d.Nkl; ++i) {
        const uint64_t r = d.storageRow[i];
        rows.push_back({static_cast<int64_t>(r % NxHalf), static_cast<int64_t>(r / NxHalf), static_cast<int32_t>(i), -1});
    }
    std::vector<int64_t> modeOfRow(NxHalf * p.Ny, -1);
    for (size_t i = 0; i < d.Nkl; ++i) modeOfRow[d.storageRow[i]] = static_cast<int64_t>(i);
    for (size_t i = 0; i < d.completionRows.size(); ++i) {
        const uint64_t r = d.completionRows[i];
        const int64_t srcMode = modeOfRow[d.completionSources[i]];
        rows.push_back({static_cast<int64_t>(r % NxHalf), static_cast<int64_t>(r / NxHalf), -1, static_cast<int32_t>(srcMode)});
    }
    std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) {
        if (a.kx != b.kx) return a.kx < b.kx;
        return a.ky < b.ky;
    });
    p.positions = rows.size();
    int64_t kxMax = 0;
    for (const auto& r : rows) kxMax = std::max(kxMax, r.kx);
    p.kxColumns = static_cast<size_t>(kxMax + 1);
    p.colStart.assign(p.kxColumns + 1, 0);
    p.posKx.resize(rows.size());
    p.posKy.resize(rows.size());
    std::vector<int32_t> posOfMode(d.Nkl, -1), compPosOfMode(d.Nkl, -1);
    for (size_t i = 0; i < rows.size(); ++i) {
        p.posKx[i] = static_cast<int32_t>(rows[i].kx);
        p.posKy[i] = static_cast<int32_t>(rows[i].ky);
        p.colStart[rows[i].kx + 1]++;
        if (rows[i].mode >= 0) posOfMode[rows[i].mode] = static_cast<int32_t>(i);
        else compPosOfMode[rows[i].compOf] = static_cast<int32_t>(i);
    }
    for (size_t k = 0; k < p.kxColumns; ++k) p.colStart[k + 1] += p.colStart[k];
    p.ymap.assign(p.kxColumns * p.Ny, -1);
    for (size_t i = 0; i < rows.size(); ++i) p.ymap[rows[i].kx * p.Ny + rows[i].ky] = static_cast<int32_t>(i);
    // Modes in position order.
    std::vector<int32_t> order(d.Nkl);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return posOfMode[a] < posOfMode[b]; });
    std::vector<uint8_t> selfRow(NxHalf * p.Ny, 0);
    for (const auto r : d.selfConjugateRows) selfRow[r] = 1;
    for (const int32_t w : order) {
        p.modeWV.push_back(w);
        p.modePos.push_back(posOfMode[w]);
        p.modeCompPos.push_back(compPosOfMode[w]);
        uint8_t flags = d.conjugated[w] ? 1 : 0;
        if (selfRow[d.storageRow[w]]) flags |= 2;
        p.modeFlags.push_back(flags);
    }
    p.rowK.resize(p.kxColumns);
    for (size_t kx = 0; kx < p.kxColumns; ++kx) p.rowK[kx] = 2.0 * kPi * (static_cast<double>(kx) / c.Lx);
    p.rowL.resize(p.Ny);
    for (size_t ky = 0; ky < p.Ny; ++ky) {
        const int64_t lm = ky <= p.Ny / 2 ? static_cast<int64_t>(ky) : static_cast<int64_t>(ky) - static_cast<int64_t>(p.Ny);
        p.rowL[ky] = 2.0 * kPi * (static_cast<double>(lm) / c.Ly);
    }

    // Vertical matrices.  Inverse (physical z <- vertical mode j), reference plan
    // semantics REDFT00 / RODFT00 with the x0.5 coefficient-production scaling
    // folded in (kernel.cpp:218-291; WVReferenceFFTEngine.cpp:88-107):
    //   cos family:  f(z_n) = 0.5 c_0 + sum_{j>=1} c_j cos(pi j n/(Nz-1))
    //   sin family:  f(z_n) = sum_{j>=1} c_j sin(pi j n/(Nz-1)),  f(z_0) = f(z_{Nz-1}) = 0
    // z-derivative channels fold -m_j (cos field -> sin) or +m_j (sin field -> cos).
    const long long L = static_cast<long long>(p.Nz) - 1;
    p.zHalf = (p.Nz + 1) / 2;
    const size_t Zh = p.zHalf, Nj = p.Nj, Nz = p.Nz;
    p.Ccos.assign(Zh * Nj, 0.0); p.Csin.assign(Zh * Nj, 0.0); p.CcosM.assign(Zh * Nj, 0.0); p.CsinM.assign(Zh * Nj, 0.0);
    for (size_t n = 0; n < Zh; ++n) {
        for (size_t j = 0; j < Nj; ++j) {
            const double cv = j == 0 ? 0.5 : cospi_ratio(static_cast<long long>(j) * static_cast<long long>(n), L);
            const double sv = (j == 0 || n == 0 || n == Nz - 1) ? 0.0 : sinpi_ratio(static_cast<long long>(j) * static_cast<long long>(n), L);
            p.Ccos[n * Nj + j] = cv;
            p.Csin[n * Nj + j] = sv;
            p.CcosM[n * Nj + j] = d.m[j] * cv;
            p.CsinM[n * Nj + j] = -d.m[j] * sv;
        }
    }
    // Forward (vertical mode j <- physical z): DCT-I / DST-I then
    // normalizeForwardDCT / normalizeForwardDST (kernel.cpp:176-193), times the
    // horizontal scale 1/(Nx Ny) of the projection (kernel.cpp:964).  Folded:
    // entry n stands for the pair (n, Nz-1-n) combined as S_n +/- S_{Nz-1-n}.
    const double inv = 1.0 / static_cast<double>(L);
    const double hs = 1.0 / static_cast<double>(p.Nx * p.Ny);
    p.Fcos.assign(Nj * Zh, 0.0); p.Fsin.assign(Nj * Zh, 0.0);
    for (size_t j = 0; j < Nj; ++j) {
        for (size_t n = 0; n < Zh; ++n) {
            double cv;
            if (n == 0) cv = 1.0;
            else cv = 2.0 * cospi_ratio(static_cast<long long>(j) * static_cast<long long>(n), L);
            double sv = (j == 0 || n == 0) ? 0.0 : 2.0 * sinpi_ratio(static_cast<long long>(j) * static_cast<long long>(n), L);
            if (j == Nz - 1) cv *= 0.5;
            p.Fcos[j * Zh + n] = cv * inv * hs;
            p.Fsin[j * Zh + n] = sv * inv * hs;
        }
    }
    const int xLen = static_cast<int>(p.Nx % 2 == 0 ? p.Nx / 2 : p.Nx);
    p.fx = factor_fft(xLen);
    p.fy = factor_fft(static_cast<int>(p.Ny));
    p.twx = twiddles(xLen);
    p.twxN = twiddles(static_cast<int>(p.Nx));
    p.twy = twiddles(static_cast<int>(p.Ny));
    if (p.Nz >= 3 && 2 * (p.Nz - 1) <= static_cast<size_t>(kMaxFFT)) {
        p.fz = factor_fft(static_cast<int>(2 * (p.Nz - 1)));
        p.twz = twiddles(static_cast<int>(2 * (p.Nz - 1)));
    }
    return {};
}

}  // namespace wvgpu
