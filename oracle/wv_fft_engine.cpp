// Test infrastructure only: O(N log N) CPU provider of the reference's
// WVFFTEngine contract (see wv_fft_engine.hpp for the definitions it computes).
//
// Every transform runs as batches of kLanes independent complex lines stored
// split (real and imaginary arrays) and interleaved by lane, x[n][lane], so the
// innermost loop of each Stockham stage runs over lanes with one twiddle.
#include "wv_fft_engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <thread>
#include <vector>

namespace wvoracle {
namespace {

using wavevortex::WVComplex64;
using wavevortex::WVFFTPlan;
using wavevortex::WVFFTPlanKind;
using wavevortex::WVFFTPlanSpecification;
using wavevortex::WVKernelStatus;
using wavevortex::WVKernelStatusCode;

constexpr std::size_t kLanes = 8;

// cos and sin of -2 pi num/den, generated in long double and rounded once.
void root(std::size_t num, std::size_t den, double& c, double& s) {
    const long double pi = 3.141592653589793238462643383279502884L;
    const long double a = -2.0L * pi * static_cast<long double>(num % den) / static_cast<long double>(den);
    c = static_cast<double>(std::cos(a));
    s = static_cast<double>(std::sin(a));
}

// Batched complex FFT of one length over kLanes lanes: Stockham autosort stages,
// e^{-2 pi i nk/N} forward, unnormalized.  Stage s with radix R and span S
// (product of the radices before it) maps in[j + r N/R] (r < R), twiddled by
// exp(-2 pi i k r/(S R)) with k = j mod S, through an R-point DFT to
// out[(j/S) S R + k + r S].
class BatchFFT {
public:
    explicit BatchFFT(std::size_t n) : n_(n) {
        std::size_t rest = n, span = 1;
        auto push = [&](std::size_t r) {
            Stage s{r, span, twr_.size(), rr_.size()};
            for (std::size_t k = 0; k < span; ++k)
                for (std::size_t q = 0; q < r; ++q) {
                    double c, si;
                    root(k * q, span * r, c, si);
                    twr_.push_back(c);
                    twi_.push_back(si);
                }
            if (r != 2 && r != 3 && r != 4)
                for (std::size_t q = 0; q < r * r; ++q) {
                    double c, si;
                    root((q / r) * (q % r), r, c, si);
                    rr_.push_back(c);
                    ri_.push_back(si);
                }
            stages_.push_back(s);
            span *= r;
            rest /= r;
        };
        while (rest % 4 == 0) push(4);
        while (rest % 2 == 0) push(2);
        while (rest % 3 == 0) push(3);
        for (std::size_t p = 5; rest > 1; p += 2)
            while (rest % p == 0) push(p);
    }

    std::size_t size() const noexcept { return n_; }

    // re/im: [n][kLanes]; wr/wi: scratch of the same size.  Result in re/im.
    void forward(double* re, double* im, double* wr, double* wi) const { run(re, im, wr, wi); }

    // inverse = conj(FFT(conj(x))), unnormalized
    void inverse(double* re, double* im, double* wr, double* wi) const {
        for (std::size_t i = 0; i < n_ * kLanes; ++i) im[i] = -im[i];
        run(re, im, wr, wi);
        for (std::size_t i = 0; i < n_ * kLanes; ++i) im[i] = -im[i];
    }

private:
    struct Stage {
        std::size_t radix, span, twiddle, roots;
    };

    template <int R>
    void stage(const Stage& s, const double* ir, const double* ii, double* orr, double* oi) const {
        const std::size_t S = s.span, stride = n_ / R;
        const double* twr = &twr_[s.twiddle];
        const double* twi = &twi_[s.twiddle];
        for (std::size_t blk = 0; blk < stride / S; ++blk) {
            for (std::size_t k = 0; k < S; ++k) {
                const std::size_t j = blk * S + k, base = blk * S * R + k;
                double cr[R], ci[R];
                for (int r = 0; r < R; ++r) {
                    cr[r] = twr[k * R + r];
                    ci[r] = twi[k * R + r];
                }
                const double* xr[R];
                const double* xi[R];
                double* yr[R];
                double* yi[R];
                for (int r = 0; r < R; ++r) {
                    xr[r] = ir + (j + r * stride) * kLanes;
                    xi[r] = ii + (j + r * stride) * kLanes;
                    yr[r] = orr + (base + r * S) * kLanes;
                    yi[r] = oi + (base + r * S) * kLanes;
                }
                for (std::size_t l = 0; l < kLanes; ++l) {
                    double vr[R], vi[R];
                    vr[0] = xr[0][l];
                    vi[0] = xi[0][l];
                    for (int r = 1; r < R; ++r) {
                        const double a = xr[r][l], b = xi[r][l];
                        vr[r] = a * cr[r] - b * ci[r];
                        vi[r] = a * ci[r] + b * cr[r];
                    }
                    if constexpr (R == 2) {
                        yr[0][l] = vr[0] + vr[1];
                        yi[0][l] = vi[0] + vi[1];
                        yr[1][l] = vr[0] - vr[1];
                        yi[1][l] = vi[0] - vi[1];
                    } else if constexpr (R == 3) {
                        const double h = 0.866025403784438646763723170752936183;  // sin(2 pi/3)
                        const double t1r = vr[1] + vr[2], t1i = vi[1] + vi[2];
                        const double t2r = vr[0] - 0.5 * t1r, t2i = vi[0] - 0.5 * t1i;
                        const double dr = vr[1] - vr[2], di = vi[1] - vi[2];
                        const double t3r = h * di, t3i = -h * dr;  // -i h d
                        yr[0][l] = vr[0] + t1r;
                        yi[0][l] = vi[0] + t1i;
                        yr[1][l] = t2r + t3r;
                        yi[1][l] = t2i + t3i;
                        yr[2][l] = t2r - t3r;
                        yi[2][l] = t2i - t3i;
                    } else {
                        static_assert(R == 4, "radix");
                        const double a0r = vr[0] + vr[2], a0i = vi[0] + vi[2];
                        const double a1r = vr[0] - vr[2], a1i = vi[0] - vi[2];
                        const double a2r = vr[1] + vr[3], a2i = vi[1] + vi[3];
                        const double a3r = vi[1] - vi[3], a3i = vr[3] - vr[1];  // -i (v1 - v3)
                        yr[0][l] = a0r + a2r;
                        yi[0][l] = a0i + a2i;
                        yr[2][l] = a0r - a2r;
                        yi[2][l] = a0i - a2i;
                        yr[1][l] = a1r + a3r;
                        yi[1][l] = a1i + a3i;
                        yr[3][l] = a1r - a3r;
                        yi[3][l] = a1i - a3i;
                    }
                }
            }
        }
    }

    // a stage of an odd prime radix: direct R-point DFT per lane
    void stageGeneric(const Stage& s, const double* ir, const double* ii, double* orr, double* oi) const {
        const std::size_t R = s.radix, S = s.span, stride = n_ / R;
        const double* twr = &twr_[s.twiddle];
        const double* twi = &twi_[s.twiddle];
        const double* wr = &rr_[s.roots];
        const double* wi = &ri_[s.roots];
        std::vector<double> vr(R), vi(R);
        for (std::size_t blk = 0; blk < stride / S; ++blk)
            for (std::size_t k = 0; k < S; ++k) {
                const std::size_t j = blk * S + k, base = blk * S * R + k;
                for (std::size_t l = 0; l < kLanes; ++l) {
                    for (std::size_t r = 0; r < R; ++r) {
                        const double a = ir[(j + r * stride) * kLanes + l], b = ii[(j + r * stride) * kLanes + l];
                        vr[r] = a * twr[k * R + r] - b * twi[k * R + r];
                        vi[r] = a * twi[k * R + r] + b * twr[k * R + r];
                    }
                    for (std::size_t a = 0; a < R; ++a) {
                        double sr = vr[0], si = vi[0];
                        for (std::size_t b = 1; b < R; ++b) {
                            sr += vr[b] * wr[a * R + b] - vi[b] * wi[a * R + b];
                            si += vr[b] * wi[a * R + b] + vi[b] * wr[a * R + b];
                        }
                        orr[(base + a * S) * kLanes + l] = sr;
                        oi[(base + a * S) * kLanes + l] = si;
                    }
                }
            }
    }

    void run(double* re, double* im, double* wr, double* wi) const {
        double* ar = re;
        double* ai = im;
        double* br = wr;
        double* bi = wi;
        for (const auto& s : stages_) {
            switch (s.radix) {
            case 4: stage<4>(s, ar, ai, br, bi); break;
            case 2: stage<2>(s, ar, ai, br, bi); break;
            case 3: stage<3>(s, ar, ai, br, bi); break;
            default: stageGeneric(s, ar, ai, br, bi);
            }
            std::swap(ar, br);
            std::swap(ai, bi);
        }
        if (ar != re) {
            std::copy(ar, ar + n_ * kLanes, re);
            std::copy(ai, ai + n_ * kLanes, im);
        }
    }

    std::size_t n_;
    std::vector<Stage> stages_;
    std::vector<double> twr_, twi_, rr_, ri_;
};

// Offsets (input, output) of every batch element, in the specification's
// batch-dimension order (first dimension outermost).
std::vector<std::pair<std::ptrdiff_t, std::ptrdiff_t>> batchOffsets(const WVFFTPlanSpecification& spec) {
    std::vector<std::pair<std::ptrdiff_t, std::ptrdiff_t>> out{{0, 0}};
    for (const auto& d : spec.batchDimensions) {
        std::vector<std::pair<std::ptrdiff_t, std::ptrdiff_t>> next;
        next.reserve(out.size() * d.count);
        for (const auto& o : out)
            for (std::size_t i = 0; i < d.count; ++i)
                next.push_back({o.first + static_cast<std::ptrdiff_t>(i) * d.inputStride,
                                o.second + static_cast<std::ptrdiff_t>(i) * d.outputStride});
        out.swap(next);
    }
    return out;
}

// Runs fn(begin, end) over [0, count) split across up to `threads` host threads
// (inline when the work is small).
template <class F>
void parallelFor(std::size_t count, unsigned threads, std::size_t workPerItem, F fn) {
    const std::size_t minWork = std::size_t(1) << 16;
    std::size_t t = std::max<std::size_t>(1, std::min<std::size_t>(threads, count));
    if (count * workPerItem < minWork * 2) t = 1;
    if (t == 1) {
        fn(std::size_t(0), count);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(t);
    for (std::size_t i = 0; i < t; ++i) {
        const std::size_t b = count * i / t, e = count * (i + 1) / t;
        pool.emplace_back([=]() { fn(b, e); });
    }
    for (auto& th : pool) th.join();
}

// 2-D r2c / c2r over groups of kLanes planes.  Planes are sorted by their offset
// on the complex side: with the reference's half-spectrum layout (z fastest,
// kernel.cpp horizontalSpecification) consecutive planes are adjacent complex
// values, so one cache line of the spectrum serves a whole group.  Columns (y)
// run one plane per lane; rows (x) carry two planes' real rows per complex
// lane, two rows per batched FFT.
class HorizontalPlan final : public WVFFTPlan {
public:
    HorizontalPlan(const WVFFTPlanSpecification& spec, unsigned threads)
        : forward_(spec.kind == WVFFTPlanKind::horizontalRealToComplex2D), threads_(threads),
          Ny_(spec.transformDimensions[0].count), Nx_(spec.transformDimensions[1].count), K_(Nx_ / 2 + 1),
          y_(spec.transformDimensions[0]), x_(spec.transformDimensions[1]), planes_(batchOffsets(spec)),
          fx_(Nx_), fy_(Ny_) {
        const bool f = forward_;
        std::stable_sort(planes_.begin(), planes_.end(), [f](const auto& a, const auto& b) {
            return f ? a.second < b.second : a.first < b.first;
        });
    }

    WVKernelStatus execute(const void* input, void* output) override {
        if (!input || !output) return {WVKernelStatusCode::invalidPointer, "Oracle FFT received a null pointer."};
        const std::size_t groups = (planes_.size() + kLanes - 1) / kLanes;
        const std::size_t work = kLanes * Nx_ * Ny_ * 8;
        parallelFor(groups, threads_, work, [&](std::size_t b, std::size_t e) {
            Scratch s(*this);
            for (std::size_t gi = b; gi < e; ++gi) {
                const std::size_t p0 = gi * kLanes, n = std::min(kLanes, planes_.size() - p0);
                if (forward_)
                    r2c(static_cast<const double*>(input), static_cast<WVComplex64*>(output), p0, n, s);
                else
                    c2r(static_cast<const WVComplex64*>(input), static_cast<double*>(output), p0, n, s);
            }
        });
        return WVKernelStatus::ok();
    }

    std::size_t persistentBytes() const noexcept override {
        return sizeof(*this) + planes_.capacity() * sizeof(planes_[0]);
    }

private:
    struct Scratch {
        explicit Scratch(const HorizontalPlan& p) {
            const std::size_t line = std::max(p.Nx_, p.Ny_) * kLanes;
            hr.resize(p.Ny_ * p.K_ * kLanes);
            hi.resize(hr.size());
            for (auto* v : {&lr, &li, &wr, &wi}) v->resize(line);
        }
        std::vector<double> hr, hi;          // [y][kx][lane]: the plane group between the two passes
        std::vector<double> lr, li, wr, wi;  // one batched line and its FFT scratch
    };

    // x rows: lane h * kLanes/2 + q carries row y + h of planes (2q, 2q + 1) as
    // re + i im; y columns: one plane per lane
    void r2c(const double* input, WVComplex64* output, std::size_t p0, std::size_t n, Scratch& s) const {
        const std::size_t half = kLanes / 2;
        for (std::size_t y = 0; y < Ny_; y += 2) {
            for (std::size_t h = 0; h < 2; ++h) {
                const std::size_t yy = y + h;
                for (std::size_t q = 0; q < half; ++q) {
                    const std::size_t ga = 2 * q, gb = 2 * q + 1, lane = h * half + q;
                    const bool rowOk = yy < Ny_;
                    const double* ra = rowOk && ga < n ? input + planes_[p0 + ga].first + static_cast<std::ptrdiff_t>(yy) * y_.inputStride : nullptr;
                    const double* rb = rowOk && gb < n ? input + planes_[p0 + gb].first + static_cast<std::ptrdiff_t>(yy) * y_.inputStride : nullptr;
                    for (std::size_t x = 0; x < Nx_; ++x) {
                        const std::ptrdiff_t o = static_cast<std::ptrdiff_t>(x) * x_.inputStride;
                        s.lr[x * kLanes + lane] = ra ? ra[o] : 0.0;
                        s.li[x * kLanes + lane] = rb ? rb[o] : 0.0;
                    }
                }
            }
            fx_.forward(s.lr.data(), s.li.data(), s.wr.data(), s.wi.data());
            // A[k] = (Z[k] + conj Z[N-k]) / 2, B[k] = (Z[k] - conj Z[N-k]) / (2 i)
            for (std::size_t h = 0; h < 2 && y + h < Ny_; ++h) {
                double* hr = &s.hr[(y + h) * K_ * kLanes];
                double* hi = &s.hi[(y + h) * K_ * kLanes];
                for (std::size_t k = 0; k < K_; ++k) {
                    const std::size_t m = (Nx_ - k) % Nx_;
                    for (std::size_t q = 0; q < half; ++q) {
                        const std::size_t lane = h * half + q;
                        const double zr = s.lr[k * kLanes + lane], zi = s.li[k * kLanes + lane];
                        const double cr = s.lr[m * kLanes + lane], ci = -s.li[m * kLanes + lane];
                        hr[k * kLanes + 2 * q] = 0.5 * (zr + cr);
                        hi[k * kLanes + 2 * q] = 0.5 * (zi + ci);
                        hr[k * kLanes + 2 * q + 1] = 0.5 * (zi - ci);
                        hi[k * kLanes + 2 * q + 1] = -0.5 * (zr - cr);
                    }
                }
            }
        }
        for (std::size_t kx = 0; kx < K_; ++kx) {
            for (std::size_t ky = 0; ky < Ny_; ++ky)
                for (std::size_t l = 0; l < kLanes; ++l) {
                    s.lr[ky * kLanes + l] = s.hr[(ky * K_ + kx) * kLanes + l];
                    s.li[ky * kLanes + l] = s.hi[(ky * K_ + kx) * kLanes + l];
                }
            fy_.forward(s.lr.data(), s.li.data(), s.wr.data(), s.wi.data());
            for (std::size_t ky = 0; ky < Ny_; ++ky) {
                const std::ptrdiff_t o = static_cast<std::ptrdiff_t>(ky) * y_.outputStride + static_cast<std::ptrdiff_t>(kx) * x_.outputStride;
                for (std::size_t g = 0; g < n; ++g) {
                    auto& v = output[planes_[p0 + g].second + o];
                    v.real = s.lr[ky * kLanes + g];
                    v.imag = s.li[ky * kLanes + g];
                }
            }
        }
    }

    // y columns (one plane per lane), then x rows with two planes per complex
    // lane; the imaginary parts of the kx = 0 and Nyquist columns do not reach
    // the output (Re of the Hermitian sum)
    void c2r(const WVComplex64* input, double* output, std::size_t p0, std::size_t n, Scratch& s) const {
        for (std::size_t kx = 0; kx < K_; ++kx) {
            for (std::size_t ky = 0; ky < Ny_; ++ky) {
                const std::ptrdiff_t o = static_cast<std::ptrdiff_t>(ky) * y_.inputStride + static_cast<std::ptrdiff_t>(kx) * x_.inputStride;
                for (std::size_t g = 0; g < kLanes; ++g) {
                    if (g < n) {
                        const auto& v = input[planes_[p0 + g].first + o];
                        s.lr[ky * kLanes + g] = v.real;
                        s.li[ky * kLanes + g] = v.imag;
                    } else {
                        s.lr[ky * kLanes + g] = s.li[ky * kLanes + g] = 0.0;
                    }
                }
            }
            fy_.inverse(s.lr.data(), s.li.data(), s.wr.data(), s.wi.data());
            for (std::size_t y = 0; y < Ny_; ++y)
                for (std::size_t l = 0; l < kLanes; ++l) {
                    s.hr[(y * K_ + kx) * kLanes + l] = s.lr[y * kLanes + l];
                    s.hi[(y * K_ + kx) * kLanes + l] = s.li[y * kLanes + l];
                }
        }
        const std::size_t half = kLanes / 2;
        const bool nyq = Nx_ % 2 == 0;
        // lane h * kLanes/2 + q carries row y + h of planes (2q, 2q + 1):
        // Z[k] = A[k] + i B[k] over their Hermitian extensions
        for (std::size_t y = 0; y < Ny_; y += 2) {
            for (std::size_t h = 0; h < 2; ++h) {
                const bool rowOk = y + h < Ny_;
                const double* hr = &s.hr[(rowOk ? y + h : y) * K_ * kLanes];
                const double* hi = &s.hi[(rowOk ? y + h : y) * K_ * kLanes];
                for (std::size_t k = 0; k < Nx_; ++k) {
                    const bool mirror = k >= K_;
                    const std::size_t src = mirror ? Nx_ - k : k;
                    const bool realOnly = k == 0 || (nyq && k == Nx_ / 2);
                    const double sg = mirror ? -1.0 : 1.0;
                    for (std::size_t q = 0; q < half; ++q) {
                        const std::size_t lane = h * half + q;
                        if (!rowOk) {
                            s.lr[k * kLanes + lane] = s.li[k * kLanes + lane] = 0.0;
                            continue;
                        }
                        const double ar = hr[src * kLanes + 2 * q], ai = realOnly ? 0.0 : sg * hi[src * kLanes + 2 * q];
                        const double br = hr[src * kLanes + 2 * q + 1], bi = realOnly ? 0.0 : sg * hi[src * kLanes + 2 * q + 1];
                        s.lr[k * kLanes + lane] = ar - bi;
                        s.li[k * kLanes + lane] = ai + br;
                    }
                }
            }
            fx_.inverse(s.lr.data(), s.li.data(), s.wr.data(), s.wi.data());
            for (std::size_t h = 0; h < 2 && y + h < Ny_; ++h)
                for (std::size_t q = 0; q < half; ++q) {
                    const std::size_t ga = 2 * q, gb = 2 * q + 1, lane = h * half + q;
                    const std::ptrdiff_t row = static_cast<std::ptrdiff_t>(y + h) * y_.outputStride;
                    double* ra = ga < n ? output + planes_[p0 + ga].second + row : nullptr;
                    double* rb = gb < n ? output + planes_[p0 + gb].second + row : nullptr;
                    for (std::size_t x = 0; x < Nx_; ++x) {
                        const std::ptrdiff_t o = static_cast<std::ptrdiff_t>(x) * x_.outputStride;
                        if (ra) ra[o] = s.lr[x * kLanes + lane];
                        if (rb) rb[o] = s.li[x * kLanes + lane];
                    }
                }
        }
    }

    bool forward_;
    unsigned threads_;
    std::size_t Ny_, Nx_, K_;
    wavevortex::WVFFTDimension y_, x_;
    std::vector<std::pair<std::ptrdiff_t, std::ptrdiff_t>> planes_;
    BatchFFT fx_, fy_;
};

// REDFT00 / RODFT00 over every batch element: two batch elements per complex
// lane (re + i im) of the even (length 2(N-1)) or odd (length 2(N+1))
// extension, kLanes lanes per batched FFT.
class VerticalPlan final : public WVFFTPlan {
public:
    VerticalPlan(const WVFFTPlanSpecification& spec, unsigned threads)
        : sine_(spec.kind == WVFFTPlanKind::verticalDSTI), threads_(threads), N_(spec.transformDimensions[0].count),
          d_(spec.transformDimensions[0]), lines_(batchOffsets(spec)),
          fft_(sine_ ? 2 * (N_ + 1) : 2 * (N_ - 1)) {}

    WVKernelStatus execute(const void* input, void* output) override {
        if (!input || !output) return {WVKernelStatusCode::invalidPointer, "Oracle FFT received a null pointer."};
        const auto* in = static_cast<const double*>(input);
        auto* out = static_cast<double*>(output);
        const std::size_t per = 2 * kLanes;  // batch elements per batched FFT
        const std::size_t groups = (lines_.size() + per - 1) / per;
        const std::size_t L = fft_.size();
        parallelFor(groups, threads_, L * kLanes * 8, [&](std::size_t b, std::size_t e) {
            std::vector<double> zr(L * kLanes), zi(L * kLanes), wr(L * kLanes), wi(L * kLanes);
            for (std::size_t gi = b; gi < e; ++gi) {
                const std::size_t e0 = gi * per;
                std::fill(zr.begin(), zr.end(), 0.0);
                std::fill(zi.begin(), zi.end(), 0.0);
                for (std::size_t q = 0; q < kLanes; ++q) {
                    const std::size_t ia = e0 + 2 * q, ib = ia + 1;
                    for (int part = 0; part < 2; ++part) {
                        const std::size_t idx = part == 0 ? ia : ib;
                        if (idx >= lines_.size()) continue;
                        double* z = part == 0 ? zr.data() : zi.data();
                        const double* src = in + lines_[idx].first;
                        if (!sine_) {
                            for (std::size_t m = 0; m < N_; ++m) {
                                const double v = src[static_cast<std::ptrdiff_t>(m) * d_.inputStride];
                                z[m * kLanes + q] = v;
                                if (m > 0 && m + 1 < N_) z[(L - m) * kLanes + q] = v;
                            }
                        } else {
                            for (std::size_t m = 0; m < N_; ++m) {
                                const double v = src[static_cast<std::ptrdiff_t>(m) * d_.inputStride];
                                z[(m + 1) * kLanes + q] = v;
                                z[(L - m - 1) * kLanes + q] = -v;
                            }
                        }
                    }
                }
                fft_.forward(zr.data(), zi.data(), wr.data(), wi.data());
                // even extension: F = DCT(a) + i DCT(b); odd: F[k+1] = -i S(a) + S(b)
                for (std::size_t q = 0; q < kLanes; ++q) {
                    const std::size_t ia = e0 + 2 * q, ib = ia + 1;
                    for (std::size_t k = 0; k < N_; ++k) {
                        const std::size_t f = sine_ ? k + 1 : k;
                        const double ya = sine_ ? -zi[f * kLanes + q] : zr[f * kLanes + q];
                        const double yb = sine_ ? zr[f * kLanes + q] : zi[f * kLanes + q];
                        if (ia < lines_.size()) out[lines_[ia].second + static_cast<std::ptrdiff_t>(k) * d_.outputStride] = ya;
                        if (ib < lines_.size()) out[lines_[ib].second + static_cast<std::ptrdiff_t>(k) * d_.outputStride] = yb;
                    }
                }
            }
        });
        return WVKernelStatus::ok();
    }

    std::size_t persistentBytes() const noexcept override {
        return sizeof(*this) + lines_.capacity() * sizeof(lines_[0]);
    }

private:
    bool sine_;
    unsigned threads_;
    std::size_t N_;
    wavevortex::WVFFTDimension d_;
    std::vector<std::pair<std::ptrdiff_t, std::ptrdiff_t>> lines_;
    BatchFFT fft_;
};

} // namespace

unsigned defaultOracleFFTThreads() {
    if (const char* env = std::getenv("WV_ORACLE_FFT_THREADS")) {
        const long v = std::strtol(env, nullptr, 10);
        if (v > 0) return static_cast<unsigned>(v);
    }
    const unsigned hw = std::thread::hardware_concurrency();
    return hw == 0 ? 1 : hw;
}

OracleFFTEngine::OracleFFTEngine(unsigned threads) : threads_(threads == 0 ? defaultOracleFFTThreads() : threads) {}

WVKernelStatus OracleFFTEngine::createPlan(const WVFFTPlanSpecification& specification, std::unique_ptr<WVFFTPlan>& plan) {
    try {
        switch (specification.kind) {
        case WVFFTPlanKind::horizontalRealToComplex2D:
        case WVFFTPlanKind::horizontalComplexToReal2D:
            if (specification.transformDimensions.size() != 2 || specification.transformDimensions[0].count == 0 ||
                specification.transformDimensions[1].count == 0)
                return {WVKernelStatusCode::invalidConfiguration, "Oracle r2c/c2r requires rank two."};
            plan = std::make_unique<HorizontalPlan>(specification, threads_);
            return WVKernelStatus::ok();
        case WVFFTPlanKind::verticalDCTI:
        case WVFFTPlanKind::verticalDSTI: {
            if (specification.transformDimensions.size() != 1)
                return {WVKernelStatusCode::invalidConfiguration, "Oracle r2r requires rank one."};
            const std::size_t n = specification.transformDimensions[0].count;
            if ((specification.kind == WVFFTPlanKind::verticalDCTI && n < 2) || n < 1)
                return {WVKernelStatusCode::invalidConfiguration, "Oracle r2r length is too short."};
            plan = std::make_unique<VerticalPlan>(specification, threads_);
            return WVKernelStatus::ok();
        }
        }
    } catch (const std::bad_alloc&) {
        return {WVKernelStatusCode::allocationFailure, "Unable to allocate an oracle FFT plan."};
    }
    return {WVKernelStatusCode::unsupportedOperation, "Unknown oracle FFT plan."};
}

} // namespace wvoracle
