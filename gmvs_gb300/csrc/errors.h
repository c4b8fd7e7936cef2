// Thread-local last-error message of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gmvs {
extern thread_local std::string g_last_error;
int32_t fail(int32_t code, const std::string& msg);
int32_t fail_cuda(cudaError_t e, const char* what);
}  // namespace gmvs
