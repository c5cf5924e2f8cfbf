// Reference include path of snncuda::core::version / cuda_available
// (include/snncuda/core/Version.h in the reference), header-only over the C
// ABI: version() is the backend's version string, cuda_available() whether a
// CUDA device can be used at run time.
#pragma once

#include <string_view>

#include "../../snncuda_gb300.h"

namespace snncuda::core {

inline std::string_view version() noexcept { return snncuda_version(); }
inline bool cuda_available() noexcept { return snncuda_cuda_available() != 0; }

}  // namespace snncuda::core
