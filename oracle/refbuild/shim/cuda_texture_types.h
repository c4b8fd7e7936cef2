/* Build shim for compiling the reference with CUDA 13, which no longer ships
 * this header; the texture types it declared live in cuda_runtime.h. */
#pragma once
#include <cuda_runtime.h>
