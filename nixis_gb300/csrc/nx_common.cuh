// nx_common.cuh -- shared definitions for the nixis_gb300 CUDA library.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/nixis_gb300.h"

#define NX_EXPORT extern "C" __attribute__((visibility("default")))

namespace nx {

// Records the message returned by nx_last_error() for this host thread.
void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);

// Number of SMs of the current device (cached per device).
int sm_count();

}  // namespace nx

#define NX_CHECK_CUDA(expr)                                   \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return nx::check_cuda(_e, #expr); \
    } while (0)

#define NX_CHECK_LAUNCH(name)                                 \
    do {                                                      \
        cudaError_t _e = cudaGetLastError();                  \
        if (_e != cudaSuccess) return nx::check_cuda(_e, name); \
    } while (0)
