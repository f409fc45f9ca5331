// Accessors of a handle for the library's other translation units (the
// handle's definition stays private to wv_api.cu).
#pragma once

#include "wvgpu.h"
#include "wv_descriptor.hpp"

#include <vector>

namespace wvgpu {

// Cap of the grid-stride element-wise launches: perSm blocks per SM of the
// current device (its multiprocessor count, queried once per device).
size_t grid_cap(size_t perSm);

const Descriptor& handle_descriptor(const wv_handle* h);
int handle_device(const wv_handle* h);
void* handle_stream(const wv_handle* h);  // the stream of the host-pointer entries
bool handle_is_single_state(const wv_handle* h);

// The handle's scheduled right-hand side (wv_evaluate_rhs_device) that also
// writes the advection fields (u, v, w) of the state, [3][Nx Ny Nz] doubles
// (evaluateRightHandSideWithContext, PortableRuntime/src/WVForcingEngine.cpp:870-895).
int scheduled_rhs_with_fields(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                              double* Fp, double* Fm, double* F0, double* fields, void* stream);

// Integration system with integrated observers (wv_system.cu), for the RK23 driver.
int system_rhs(wv_system* s, double t, double t0, const double* state, double* rhs, void* stream);
size_t system_extra_doubles(const wv_system* s);
const double* system_extra_tolerances(const wv_system* s);  // device [extra]
wv_handle* system_handle(const wv_system* s);
void system_blocks(const wv_system* s, std::vector<uint64_t>& lengths, std::vector<double>& tolerances);

}  // namespace wvgpu
