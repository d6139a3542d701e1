// launch_fp32.cu -- FP32 kernel instantiations (multiply-adds contracted
// into FMAs).
#define MCV_DEFINE_LAUNCHERS
#include "kernels.cuh"

template struct mcv::Launchers<float>;
