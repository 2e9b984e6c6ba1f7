// Launcher of the off-grid marginal kernels (offgrid.cu), called by the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "pdq.h"
#include "pdq_device.cuh"

cudaError_t pdq_launch_offgrid(const pdq_offgrid_args& a, const double (&q1)[pdq::kMaxN][pdq::kMaxN],
                               cudaStream_t stream);
