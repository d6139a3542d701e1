// launch_fp64.cu -- FP64 kernel instantiations.  Compiled with
// --fmad=false: every multiply and add rounds separately, as in the CPU
// restatement (compiled with -ffp-contract=off), so FP64 results agree with
// it operation for operation and differ only where the math libraries'
// transcendental functions do.
#define MCV_DEFINE_LAUNCHERS
#include "kernels.cuh"

template struct mcv::Launchers<double>;
