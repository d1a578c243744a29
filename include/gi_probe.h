/*
 * gi_probe.h - device peak probe of the GB300 line-intensity engine.
 *
 * The roofline denominators of the FP64 path are not in the driver-written
 * peak table (it holds HBM copy bandwidth and bf16 GEMM throughput), so the
 * engine measures the FP64 tensor-pipe peak itself: a kernel that issues only
 * independent mma.sync m8n8k4 .f64 instructions on every SM.  No counterpart
 * in the reference (it has no performance instrumentation beyond wall time,
 * main.cu:91-93).
 */
#ifndef GI_PROBE_H
#define GI_PROBE_H
#include "gi.h"
#ifdef __cplusplus
extern "C" {
#endif
/* Measured FP64 DMMA throughput of `device` in TFLOP/s (best of 3). */
gi_status gi_measure_fp64_peak(int device, double* tflops);
#ifdef __cplusplus
}
#endif
#endif
