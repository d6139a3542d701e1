/*
 * acc_gb300_probe.h -- measurement probes (no reference counterpart).
 *
 * The propagation kernels are bound by the FP32/FP64 pipes, the
 * special-function unit and L2 atomics, none of which the driver-measured
 * peak file records; these
 * probes measure them on the running GPU so that a roofline fraction can
 * be quoted against a measured peak.
 */
#ifndef ACC_GB300_PROBE_H
#define ACC_GB300_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Dense FMA throughput of the FP32 (precision 32) or FP64 (64) pipe on
 * `device`, in TFLOP/s (2 flops per FMA), best of `repeats` launches of
 * about 20 ms each. */
int mcv_probe_fma_peak(int device, int precision, int repeats, double* tflops);

/* Special-function-unit throughput on `device` (FP32 base-2 exponentials,
 * ex2.approx), in operations per second, best of `repeats` launches. */
int mcv_probe_sfu_rate(int device, int repeats, double* ops_per_s);

/* FP64 atomicAdd throughput into `nbins` distinct doubles of a
 * device-resident histogram (addresses hashed from the thread index), in
 * atomic operations per second, best of `repeats`. */
int mcv_probe_atomic_rate(int device, uint64_t nbins, int repeats,
                          double* ops_per_s);

#ifdef __cplusplus
}
#endif

#endif
