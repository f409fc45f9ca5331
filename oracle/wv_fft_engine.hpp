// Test infrastructure only (oracle side): an O(N log N) CPU provider of the
// reference's FFT engine contract, so that the reference's own C++ kernel and
// runtime (built by oracle/ref_build.sh) can run at 256x256x129-class grids.
// The reference's own providers are FFTW 3.3.11 (absent from this image) and a
// direct O(N^4) DFT (adapters/reference/WVReferenceFFTEngine.cpp), which is
// exact but infeasible beyond ~32x32x17.  The shipped GPU library never links
// or loads this file.
//
// Contract implemented: CompiledKernel/include/WaveVortexKernel/WVFFTEngine.hpp:41-50
// (createPlan over WVFFTPlanSpecification, guru-style strided transform and
// batch dimensions).  Transform definitions, as the direct engine states them
// (CompiledKernel/adapters/reference/WVReferenceFFTEngine.cpp:47-107) and as
// FFTW defines them:
//   r2c 2-D   X[ky,kx] = sum_{y,x} x[y,x] e^{-2 pi i (kx x/Nx + ky y/Ny)}, kx <= Nx/2
//   c2r 2-D   x[y,x]   = Re sum over the Hermitian extension of X, unnormalized
//   REDFT00   y[k] = x[0] + (-1)^k x[N-1] + 2 sum_{n=1}^{N-2} x[n] cos(pi n k/(N-1))
//   RODFT00   y[k] = 2 sum_{n=0}^{N-1} x[n] sin(pi (n+1)(k+1)/(N+1))
// computed with mixed-radix Stockham FFTs (radix 4, 2, 3, 5 and a direct
// odd-prime stage); REDFT00 / RODFT00 as complex FFTs of the even / odd
// extension of length 2(N-1) / 2(N+1), two real transforms of one batch per
// complex line; real rows of the 2-D transforms likewise two per complex line.
// Work is split over the batch across host threads (WV_ORACLE_FFT_THREADS,
// default: every hardware thread).
#pragma once

#include "WaveVortexKernel/WVFFTEngine.hpp"

#include <memory>
#include <string>

namespace wvoracle {

class OracleFFTEngine final : public wavevortex::WVFFTEngine {
public:
    // threads == 0: WV_ORACLE_FFT_THREADS if set, else std::thread::hardware_concurrency()
    explicit OracleFFTEngine(unsigned threads = 0);
    std::string identifier() const override { return "oracle-stockham"; }
    std::size_t persistentBytes() const noexcept override { return sizeof(*this); }
    wavevortex::WVKernelStatus createPlan(const wavevortex::WVFFTPlanSpecification& specification,
                                          std::unique_ptr<wavevortex::WVFFTPlan>& plan) override;
    unsigned threads() const noexcept { return threads_; }

private:
    unsigned threads_;
};

// Threads a default-constructed engine uses.
unsigned defaultOracleFFTThreads();

} // namespace wvoracle
