// Accessors of a handle for the library's other translation units (the
// handle's definition stays private to wv_api.cu).
#pragma once

#include "wvgpu.h"
#include "wv_descriptor.hpp"

namespace wvgpu {

const Descriptor& handle_descriptor(const wv_handle* h);
int handle_device(const wv_handle* h);
void* handle_stream(const wv_handle* h);  // the stream of the host-pointer entries
bool handle_is_single_state(const wv_handle* h);

}  // namespace wvgpu
