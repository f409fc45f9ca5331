// Device layout plan of one handle: which half-spectrum rows carry data,
// their order in HBM, the vertical transform matrices with all reference
// normalizations folded in, FFT factorizations and twiddles.
//
// Layouts in HBM (T = double for FP64 handles, float for MIXED):
//   zspec   [ch][z][pos]          vertical-inverse output, pos = active row in (kx, ky) order
//   yspec   [z][ch][y][kx]        after the inverse y FFTs (kx < kxColumns)
//   pspec   [z][q][y][kx]         r2c of the quadratic products along x (kx < kxColumns)
//   fspec   [q][z][pos]           after the forward y FFTs, gathered to active rows
// Only kx < kxColumns and the active rows are ever touched: the 2/3 disk
// makes every other row of the half spectrum identically zero.
#pragma once

#include "wv_descriptor.hpp"

#include <cstdint>
#include <vector>

namespace wvgpu {

constexpr int kMaxStages = 24;
constexpr int kMaxFFT = 1024;

struct FFTFactors {
    int N = 0;
    int nstages = 0;
    int radix[kMaxStages] = {};
};

FFTFactors factor_fft(int N);

// Targets of the nonlinear flux: 0=u, 1=v, 2=w, 3=eta.
struct TargetSet {
    int count = 0;
    int q[4] = {};
};

struct Plan {
    size_t Nx = 0, Ny = 0, Nz = 0, Nj = 0, Nkl = 0, NxHalf = 0, M = 0;
    size_t positions = 0;     // active rows (retained + completion)
    size_t kxColumns = 0;     // kx < kxColumns hold data
    size_t zHalf = 0;         // (Nz+1)/2 rows of the folded vertical matrices
    TargetSet targets;        // {u,v,w,eta} nonhydrostatic, {u,v,eta} hydrostatic
    // Active rows in (kx, ky) order.
    std::vector<int32_t> posKx, posKy;
    std::vector<int32_t> colStart;        // [kxColumns+1] positions of each kx column
    std::vector<int32_t> ymap;            // [kxColumns][Ny] position of row (kx, ky), -1 if inactive
    // Modes (retained WV columns) in position order.
    std::vector<int32_t> modeWV;          // WV index
    std::vector<int32_t> modePos;         // position of its storage row
    std::vector<int32_t> modeCompPos;     // position of its Hermitian completion row, -1 if none
    std::vector<uint8_t> modeFlags;       // bit0: stored conjugated; bit1: self-conjugate row
    // Per position wavenumbers of the stored row.
    std::vector<double> rowK;             // [kxColumns]  2*pi*kx/Lx
    std::vector<double> rowL;             // [Ny]         2*pi*lMode(ky)/Ly
    // Vertical matrices, folded by the z <-> Nz-1-z symmetry: [zHalf][Nj].
    std::vector<double> Ccos, Csin, CcosM, CsinM;
    // Forward matrices [Nj][zHalf] with 1/(Nz-1) (and 1/(Nx Ny)) folded in.
    std::vector<double> Fcos, Fsin;
    FFTFactors fx, fy;                    // fx: x line length (Nx/2 for even Nx, else Nx)
    std::vector<double> twx, twxN, twy;   // interleaved exp(-2 pi i k / N) for the x line, Nx, Ny
    // Vertical transforms as FFTs of the even / odd extension over z: length
    // 2 (Nz - 1) (0 when Nz < 3) and its twiddles.
    FFTFactors fz;
    std::vector<double> twz;
    // FFT variant per axis: the shared-memory Stockham kernels instead of the
    // register-resident warp FFTs where both exist (set by the ensemble autotuner).
    bool stockhamY = false, stockhamX = false;
};

Status build_plan(const Descriptor& d, Plan& p);

}  // namespace wvgpu
