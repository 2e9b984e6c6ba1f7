/*
 * pdq_probe.h -- measurement helpers of the GB300 build.
 *
 * These functions have no counterpart in the reference (which publishes no
 * performance numbers); they exist so the benchmark can state the FP32
 * CUDA-core roofline it reports against.
 */
#ifndef PDQ_PROBE_H_
#define PDQ_PROBE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Launch an FP32 FMA-throughput kernel: `blocks` x `threads` threads, each
 * running `iters` iterations of 8 independent FMA chains (16 flops per
 * iteration per chain pair); writes one float per thread to `out` (device,
 * blocks*threads floats) so the work cannot be eliminated.  FLOPs performed =
 * blocks * threads * iters * 16.  Asynchronous on `stream`.  Returns 0 on
 * success, 3 on a launch error. */
int pdq_probe_fp32_fma(float* out, int64_t iters, int32_t blocks, int32_t threads, void* stream);

/* Number of streaming multiprocessors of the current device (0 on error). */
int pdq_probe_sm_count(void);

#ifdef __cplusplus
}
#endif

#endif /* PDQ_PROBE_H_ */
