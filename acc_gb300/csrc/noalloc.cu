// noalloc.cu -- mcv_run_batched_noalloc: the batched launch of
// mcv_run_batched with its scratch (the staged variant descriptions and the
// counters / work-queue head) in a static device array instead of memory a
// context allocates.  It makes no allocation of its own, for callers that
// must not allocate device memory: a plugin inside a host application that
// hands out every byte of device memory from its own pool and accounts for
// it, or a caller that cannot take the device-wide synchronisation of
// freeing and re-allocating a growing staging buffer (mcv_run_batched grows
// its staging with cudaStreamSynchronize, cudaFree and cudaMalloc).

#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.cuh"

extern template struct mcv::Launchers<float>;
extern template struct mcv::Launchers<double>;

namespace {

using mcv::DevStatus;

constexpr size_t kStatusBytes = 256;  // DevStatus, padded to the alignment
constexpr size_t kChainsBytes =
    (size_t)MCV_NOALLOC_MAX_VARIANTS * sizeof(mcv_chain);
constexpr size_t kCountBytes = (size_t)MCV_NOALLOC_MAX_VARIANTS * 8;
constexpr size_t kScratchBytes =
    kStatusBytes + kChainsBytes + 2 * kCountBytes;
static_assert(sizeof(DevStatus) <= kStatusBytes, "status region too small");
static_assert(kChainsBytes % 8 == 0, "chain array must keep 8-byte alignment");

// The scratch: [DevStatus | variants[64] | counts[64] | seeds[64]].  Every
// GPU that loads the library holds it until the process exits; every call
// shares it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};

void set_msg(mcv_status* st, int code, const char* msg) {
  if (!st) return;
  st->code = code;
  snprintf(st->message, sizeof st->message, "%s", msg);
}

// Device address of the scratch on the current device; looked up on the
// first call per device (the array's name is only a host-side stand-in).
// The address belongs to the device's primary context; a cudaDeviceReset
// would end it, and the header rules out calls after one.
int scratch_on_current_device(unsigned char** out, mcv_status* st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_msg(st, MCV_ENODEV, "mcv_run_batched_noalloc: no usable CUDA device");
    return MCV_ENODEV;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      set_msg(st, MCV_ECUDA,
              "mcv_run_batched_noalloc: cudaGetSymbolAddress failed");
      return MCV_ECUDA;
    }
    g_scratch_addr[dev] = (unsigned char*)p;
  }
  *out = g_scratch_addr[dev];
  return MCV_OK;
}

// the launch shape of mcv_run_batched: up to 256 threads a block, blocks =
// SMs x resident blocks, work items of 8192 neutrons
template <typename R>
void launch_from_scratch(unsigned char* scratch, int nvar,
                         const mcv_launch* launch, cudaStream_t s) {
  DevStatus* status = (DevStatus*)scratch;
  const mcv_chain* chains = (const mcv_chain*)(scratch + kStatusBytes);
  const uint64_t* counts =
      (const uint64_t*)(scratch + kStatusBytes + kChainsBytes);
  const uint64_t* seeds = counts + MCV_NOALLOC_MAX_VARIANTS;
  int t = (launch && launch->threads_per_block > 0) ? launch->threads_per_block
                                                    : mcv::kMaxThreads;
  if (t > mcv::kMaxThreads) t = mcv::kMaxThreads;
  t = (t + 31) / 32 * 32;
  size_t smem = (sizeof(mcv_chain) + 15) / 16 * 16 + 8 * (size_t)(nvar + 1);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int blocks = (launch && launch->blocks > 0)
                   ? launch->blocks
                   : sms * mcv::Launchers<R>::occupancy_batched(t, smem);
  uint64_t chunk = (launch && launch->chunk > 0) ? (uint64_t)launch->chunk
                                                 : 8192;
  mcv::Launchers<R>::batched(blocks, t, smem, s, chains, nvar, counts, seeds,
                             chunk, status);
}

}  // namespace

extern "C" int mcv_run_batched_noalloc(const mcv_chain* variants,
                                       int32_t nvariants,
                                       const uint64_t* counts,
                                       const uint64_t* seeds, int precision,
                                       const mcv_launch* launch, void* stream,
                                       mcv_status* st) {
  if (!variants || !counts || !seeds || nvariants < 1) {
    set_msg(st, MCV_EINVAL, "mcv_run_batched_noalloc: need >= 1 variant");
    return MCV_EINVAL;
  }
  if (nvariants > MCV_NOALLOC_MAX_VARIANTS) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "mcv_run_batched_noalloc: %d variants exceed the static scratch "
             "maximum of %d",
             (int)nvariants, MCV_NOALLOC_MAX_VARIANTS);
    set_msg(st, MCV_ECAPACITY, msg);
    return MCV_ECAPACITY;
  }
  if (precision != MCV_FP32 && precision != MCV_FP64) {
    set_msg(st, MCV_EINVAL, "mcv_run_batched_noalloc: precision must be 32 "
                            "or 64");
    return MCV_EINVAL;
  }
  for (int v = 0; v < nvariants; ++v) {
    int rc = mcv::validate_chain_for(variants + v, st);
    if (rc) {
      if (st) st->first_bad_component = v;
      return rc;
    }
  }
  unsigned char* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch, st);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the previous call's contents stay in the array: clear the counters and
  // the work-queue head, overwrite the descriptions
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(DevStatus), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kStatusBytes, variants,
                        (size_t)nvariants * sizeof(mcv_chain),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kStatusBytes + kChainsBytes, counts,
                        (size_t)nvariants * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kStatusBytes + kChainsBytes + kCountBytes,
                        seeds, (size_t)nvariants * 8, cudaMemcpyHostToDevice,
                        s);
  if (e != cudaSuccess) {
    set_msg(st, MCV_ECUDA, "mcv_run_batched_noalloc: staging copy failed");
    return MCV_ECUDA;
  }
  if (precision == MCV_FP32)
    launch_from_scratch<float>(scratch, nvariants, launch, s);
  else
    launch_from_scratch<double>(scratch, nvariants, launch, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_msg(st, MCV_ECUDA, "mcv_run_batched_noalloc: launch failed");
    return MCV_ECUDA;
  }
  if (!st) return MCV_OK;
  DevStatus h;
  e = cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_msg(st, MCV_ECUDA, "mcv_run_batched_noalloc: kernel execution failed");
    return MCV_ECUDA;
  }
  uint64_t expected = 0;
  for (int v = 0; v < nvariants; ++v) expected += counts[v];
  st->code = MCV_OK;
  st->message[0] = 0;
  st->processed = h.processed;
  st->bounce_overflow = h.bounce_overflow;
  st->nonfinite = h.nonfinite;
  st->bin_oob = h.bin_oob;
  if (h.processed != expected) {
    set_msg(st, MCV_ECOUNT,
            "mcv_run_batched_noalloc: processed neutron count does not match");
    return MCV_ECOUNT;
  }
  if (h.bounce_overflow) {
    set_msg(st, MCV_EBOUNCE,
            "mcv_run_batched_noalloc: neutrons reached the guide bounce "
            "limit");
    return MCV_EBOUNCE;
  }
  return MCV_OK;
}
