// launch_fp64.cu -- FP64 kernel instantiations.  Compiled with
// --fmad=false: every multiply and add rounds separately, as in the CPU
// restatement (compiled with -ffp-contract=off), so FP64 results agree with
// it operation for operation and differ only where the math libraries'
// transcendental functions do.
#define MCV_DEFINE_LAUNCHERS
#include "kernels.cuh"

template struct mcv::Launchers<double>;

namespace mcv {
// dL/d s_j = sum over K > j of powder_x[K] + powder_y[j]: the reachable
// peaks of a neutron are a prefix of the q-sorted list.
__global__ void powder_grad_finalize(const double* powder_x,
                                     const double* powder_y, int npeaks,
                                     double* dtable) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double suffix = 0.0;
  for (int j = npeaks - 1; j >= 0; --j) {
    suffix += powder_x[j + 1];
    dtable[j] += suffix + powder_y[j];
  }
}

}  // namespace mcv

void mcv::powder_finalize(const double* px, const double* py, int npeaks,
                          double* dtable, cudaStream_t s) {
  powder_grad_finalize<<<1, 1, 0, s>>>(px, py, npeaks, dtable);
}
