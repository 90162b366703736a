// common.cuh -- shared types and helpers of the emida GB300 kernels.
//
// Types mirror the reference's ABI-visible ones (src/common.hpp:24-145):
// positions are pairs of uint32 (x, y), the argmax result is {T value; uint32 index}.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

namespace emida_gb {

using esize_t = uint32_t;

// src/common.hpp:152-159 data_index<T>: {T data; esize_t index;}
template <typename T>
struct data_index {
    T data;
    esize_t index;
};

struct size2 {
    esize_t x, y;
};

__host__ __device__ inline esize_t div_up(esize_t a, esize_t b) { return (a + b - 1) / b; }

enum policy_t : int32_t { POLICY_BRUTE = 0, POLICY_FFT = 1 };

// Status codes of the C ABI (include/emida_gb.h).
enum status_t : int32_t {
    ST_OK = 0,
    ST_INVALID_ARGUMENT = -1,
    ST_CUDA = -2,
    ST_UNSUPPORTED = -3,
    ST_DEVICE_CHECK = -4,
    ST_OUT_OF_MEMORY = -5,
};

// Device-side error word bits, set by kernels that detect a bad index or a
// bounded wait that ran out.  The host reads it after a launch sequence.
enum dev_err_t : uint32_t {
    DEV_ERR_TMA_TIMEOUT = 1u,
    DEV_ERR_BAD_INDEX = 2u,
    DEV_ERR_WAIT_TIMEOUT = 4u,  // a pipeline wait (mbarrier) ran out
};

}  // namespace emida_gb
