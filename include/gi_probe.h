/*
 * gi_probe.h - device peak probe of the GB300 line-intensity engine.
 *
 * The FP64 path's roofline denominator is not in the measured peak table
 * (that holds HBM copy bandwidth and bf16 GEMM throughput), so the engine
 * measures the FP64 tensor-pipe peak itself: a kernel that issues only
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
/* The split-precision GEMM alone on host arrays, for tests on arbitrary
   operands: C[n*M + m] = sum_k A[m*K + k] * B[n*K + k] with `slices` bf16
   digits per operand (0: the engine's default), on the kernel that the
   engine's tuner table or GI_SPLIT_FORCE selects for the shape. */
gi_status gi_probe_split_gemm(int device, int slices, int M, int N, int K, const double* A,
                              const double* B, double* C);
#ifdef __cplusplus
}
#endif
#endif
