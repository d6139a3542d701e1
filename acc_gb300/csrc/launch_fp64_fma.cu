// launch_fp64_fma.cu -- the FP64 fused chain kernel compiled with nvcc's
// default multiply-add contraction.
//
// launch_fp64.cu builds the FP64 kernels with --fmad=false, so that they
// agree with the CPU restatement operation for operation; that costs FP64
// throughput.  This unit gives a caller that asks for it
// (mcv_launch.variant == MCV_VARIANT_FP64_FMA in mcv_run_chain) the same
// kernel with contracted multiply-adds.  It is compiled with -Dmcv=mcv_fma,
// so that its kernels, device functions and launchers are symbols of their
// own; only the entry points below are seen by engine.cu.
#include "kernels.cuh"

int mcv_fp64_fma_occupancy(int x, int threads) {
  return x ? mcv::occupancy_of(mcv::chain_kernel<double, 0, true>, threads, 0)
           : mcv::occupancy_of(mcv::chain_kernel<double, 0, false>, threads,
                               0);
}

void mcv_fp64_fma_chain(int x, int blocks, int threads, cudaStream_t s,
                        const mcv_chain& ch, uint64_t n, uint64_t first,
                        uint64_t seed, void* status) {
  auto* st = static_cast<mcv::DevStatus*>(status);
  if (x)
    mcv::chain_kernel<double, 0, true><<<blocks, threads, 0, s>>>(
        ch, n, first, seed, nullptr, 0, nullptr, nullptr, st);
  else
    mcv::chain_kernel<double, 0, false><<<blocks, threads, 0, s>>>(
        ch, n, first, seed, nullptr, 0, nullptr, nullptr, st);
}

// the multiple-scattering tree kernel
int mcv_fp64_fma_ms_occupancy(int threads) {
  return mcv::occupancy_of(mcv::ms_chain_kernel<double>, threads, 0);
}

void mcv_fp64_fma_ms(int blocks, int threads, cudaStream_t s,
                     const mcv_chain& ch, uint64_t n, uint64_t first,
                     uint64_t seed, void* status) {
  auto* st = static_cast<mcv::DevStatus*>(status);
  mcv::ms_chain_kernel<double><<<blocks, threads, 0, s>>>(ch, n, first, seed,
                                                          st);
}
