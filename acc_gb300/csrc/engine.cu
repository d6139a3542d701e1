// engine.cu -- the extern "C" entry points declared in include/acc_gb300.h
// (host side; the kernels are instantiated in launch_fp32.cu and
// launch_fp64.cu).

#include <cstdio>
#include <cstring>
#include <new>

#include "kernels.cuh"

extern template struct mcv::Launchers<float>;
extern template struct mcv::Launchers<double>;

// launch_fp64_fma.cu: the FP64 chain kernel with contracted multiply-adds
int mcv_fp64_fma_occupancy(int x, int threads);
void mcv_fp64_fma_chain(int x, int blocks, int threads, cudaStream_t s,
                        const mcv_chain& ch, uint64_t n, uint64_t first,
                        uint64_t seed, void* status);
int mcv_fp64_fma_ms_occupancy(int threads);
void mcv_fp64_fma_ms(int blocks, int threads, cudaStream_t s,
                     const mcv_chain& ch, uint64_t n, uint64_t first,
                     uint64_t seed, void* status);

// =================================================================== host
using namespace mcv;

struct mcv_ctx {
  int device;
  int sm_count;
  DevStatus* d_status;
  void* d_batch;        // staged variant descriptions (mcv_run_batched)
  size_t batch_bytes;
  double* d_grad;       // powder gradient partial sums (mcv_backward)
  size_t grad_bytes;
};

struct mcv_graph {
  mcv_ctx* ctx;
  void* d_batch;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

namespace {

void set_msg(mcv_status* st, int code, const char* fmt, const char* a = "",
             long long b = 0) {
  if (!st) return;
  st->code = code;
  snprintf(st->message, sizeof st->message, fmt, a, b);
}

int cuda_fail(mcv_status* st, cudaError_t e, const char* where) {
  set_msg(st, MCV_ECUDA, "%s: CUDA error %lld", where, (long long)e);
  if (st) {
    size_t l = strlen(st->message);
    snprintf(st->message + l, sizeof st->message - l, " (%s)",
             cudaGetErrorString(e));
  }
  return MCV_ECUDA;
}

class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev_);
    if (prev_ != dev) cudaSetDevice(dev);
    dev_ = dev;
  }
  ~DeviceGuard() {
    if (prev_ != dev_) cudaSetDevice(prev_);
  }

 private:
  int prev_ = 0, dev_ = 0;
};

// The parameters of one scattering kernel (an HSS / HMS component's, or a
// composite kernel's element, whose kind may not be composite itself).
int validate_kernel(const mcv_component& c, int ker, int64_t k,
                    bool composite_ok, mcv_status* st) {
  if (ker == MCV_KERNEL_POWDER &&
      (!c.table || !c.ftable || c.ip[4] < 1 || c.dp[10] <= 0)) {
    set_msg(st, MCV_EINVAL, "component %s%lld: powder kernel needs peaks", "",
            (long long)k);
    return MCV_EINVAL;
  }
  if (ker == MCV_KERNEL_SQE_GRID &&
      (!c.ftable || c.ip[4] < 2 || c.ip[5] < 2)) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: S(Q,E) kernel needs a >= 2x2 table", "",
            (long long)k);
    return MCV_EINVAL;
  }
  if (ker == MCV_KERNEL_E_Q &&
      (!c.table || !c.ftable || c.ip[4] < 1 || c.ip[4] > MCV_EXPR_MAX_OPS ||
       c.ip[5] < 1 || c.ip[5] > MCV_EXPR_MAX_OPS || !(c.dp[12] >= 1) ||
       !(c.dp[12] <= 1e6))) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: E(Q) kernel needs E(Q) and S(Q) programs of "
            "1..256 instructions and 1 <= max_iter <= 1e6",
            "", (long long)k);
    return MCV_EINVAL;
  }
  if (ker == MCV_KERNEL_SANS2D &&
      (!c.table || !c.ftable || c.ip[4] < 2 || c.ip[5] < 2 ||
       !(c.dp[11] > c.dp[10]) || !(c.dp[13] > c.dp[12]))) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: SANS2D kernel needs a >= 2x2 S(Qx, Qy) grid "
            "over increasing Q ranges", "", (long long)k);
    return MCV_EINVAL;
  }
  if (ker == MCV_KERNEL_COMPOSITE &&
      (!composite_ok || c.ip[4] < 1 || c.ip[4] > MCV_COMPOSITE_MAX)) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: a composite kernel holds 1..16 elements, none "
            "of them composite", "", (long long)k);
    return MCV_EINVAL;
  }
  if (ker == MCV_KERNEL_DGSSXRES && !(c.dp[20] >= 0)) {
    set_msg(st, MCV_EINVAL, "component %s%lld: DGSSXRes kernel needs dtof >= 0",
            "", (long long)k);
    return MCV_EINVAL;
  }
  if (ker < MCV_KERNEL_ISOTROPIC || ker > MCV_KERNEL_DGSSXRES) {
    set_msg(st, MCV_EINVAL, "component %s%lld: unknown scattering kernel", "",
            (long long)k);
    return MCV_EINVAL;
  }
  return MCV_OK;
}

// A composite kernel at slot k: its N elements fill the next N slots,
// each a kernel element of a non-composite kind with a positive weight
// and running sums that increase to 1.
int validate_composite(const mcv_chain* ch, int k, mcv_status* st) {
  const int n = ch->comp[k].ip[4];
  if (k + n >= ch->ncomp) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: a composite kernel's elements must follow it "
            "in the chain", "", (long long)k);
    return MCV_EINVAL;
  }
  double run = 0.0;
  for (int i = 1; i <= n; ++i) {
    const mcv_component& e = ch->comp[k + i];
    const double w = e.dp[22], cum = e.dp[23];
    if (e.opcode != MCV_OP_KERNEL_ELEMENT || !(w > 0) ||
        !(fabs(cum - (run + w)) <= 1e-9) || !(cum <= 1.0 + 1e-9)) {
      set_msg(st, MCV_EINVAL,
              "component %s%lld: composite kernel element with a bad slot, "
              "weight or running weight", "", (long long)(k + i));
      return MCV_EINVAL;
    }
    run = cum;
    int rc = validate_kernel(e, e.ip[1], k + i, false, st);
    if (rc) return rc;
  }
  if (!(fabs(run - 1.0) <= 1e-9)) {
    set_msg(st, MCV_EINVAL,
            "component %s%lld: composite kernel weights must sum to 1", "",
            (long long)k);
    return MCV_EINVAL;
  }
  return MCV_OK;
}

int validate_component(const mcv_component& c, int k, mcv_status* st) {
  if (c.opcode < 0 || c.opcode >= MCV_OP_COUNT) {
    set_msg(st, MCV_EINVAL, "component %s%lld: unknown opcode", "",
            (long long)k);
    return MCV_EINVAL;
  }
  switch (c.opcode) {
    case MCV_OP_PSD_MONITOR:
    case MCV_OP_PSD_MONITOR_4PI:
    case MCV_OP_POSDIV_MONITOR:
    case MCV_OP_IQE_MONITOR:
    case MCV_OP_THETA_TOF_4PI:
    case MCV_OP_CYL_IQE_DETECTOR:
      if (c.ip[0] < 1 || c.ip[1] < 1) {
        set_msg(st, MCV_EINVAL, "component %s%lld: bin counts must be >= 1",
                "", (long long)k);
        return MCV_EINVAL;
      }
      break;
    case MCV_OP_WAVELENGTH_MONITOR:
    case MCV_OP_ENERGY_MONITOR:
      if (c.ip[0] < 1) {
        set_msg(st, MCV_EINVAL, "component %s%lld: bin count must be >= 1", "",
                (long long)k);
        return MCV_EINVAL;
      }
      break;
    case MCV_OP_BANKED_DETECTOR:
      if (c.ip[0] < 1 || c.ip[1] < 1 || c.ip[2] < 1 || c.ip[3] < 1) {
        set_msg(st, MCV_EINVAL, "component %s%lld: bin counts must be >= 1",
                "", (long long)k);
        return MCV_EINVAL;
      }
      break;
    case MCV_OP_NEUTRON_TO_STORAGE:
      if (!c.tally || c.table_len < 1) {
        set_msg(st, MCV_EINVAL,
                "component %s%lld: neutron storage needs a buffer of >= 1 "
                "rows", "", (long long)k);
        return MCV_EINVAL;
      }
      break;
    case MCV_OP_NEUTRON_STORAGE:
      if (!c.table || !c.ftable || c.table_len < 10 || c.table_len % 10) {
        set_msg(st, MCV_EINVAL,
                "component %s%lld: stored neutrons need an N x 10 table", "",
                (long long)k);
        return MCV_EINVAL;
      }
      break;
    case MCV_OP_SNS_SOURCE: {
      const int nE = c.ip[1], nt = c.ip[2];
      const bool ok = c.table && nE >= 3 && nt >= 3 &&
                      c.table_len >= (uint64_t)(2 * nE + nt) +
                                         (uint64_t)nE * nt &&
                      c.ip[3] >= 1 && c.ip[3] < nE && c.ip[4] >= 1 &&
                      c.ip[4] < nE && c.ip[5] >= 0 && c.ip[6] >= 1 &&
                      c.ip[6] <= nt && c.ip[5] < c.ip[6] && c.dp[5] > 0 &&
                      c.dp[18] >= 0 && c.dp[19] >= 0 &&
                      c.dp[18] + c.dp[19] <= MCV_SNS_TAIL_MAX &&
                      c.dp[18] == floor(c.dp[18]) &&
                      c.dp[19] == floor(c.dp[19]);
      if (!ok) {
        set_msg(st, MCV_EINVAL,
                "component %s%lld: SNS source needs its E / t tables "
                "(>= 3 points each), index ranges inside them and at most "
                "MCV_SNS_TAIL_MAX tail energies",
                "", (long long)k);
        return MCV_EINVAL;
      }
      break;
    }
    case MCV_OP_GUIDE_ANYSHAPE: {
      const int nf = c.ip[0], nv = c.ip[1];
      if (nf < 1 || nf > MCV_ANYSHAPE_MAX_FACES || nv < 3 ||
          nv > MCV_ANYSHAPE_MAX_VERTICES || !c.table || !c.ftable ||
          c.table_len < (uint64_t)nf * (12 + 2 * nv)) {
        set_msg(st, MCV_EINVAL,
                "component %s%lld: mesh guide needs 1..99 faces of 3..16 "
                "vertices and its face table", "", (long long)k);
        return MCV_EINVAL;
      }
      break;
    }
    case MCV_OP_GUIDE_TAPERING: {
      const uint64_t nblk =
          c.ip[1] > 0 ? ((uint64_t)c.ip[0] + c.ip[1] - 1) / c.ip[1] : 0;
      if (c.ip[0] < 1 || !c.table || !c.ftable || c.ip[1] < 0 ||
          c.table_len < (uint64_t)10 * c.ip[0] + 2 * nblk ||
          !(c.dp[0] > 0)) {
        set_msg(st, MCV_EINVAL,
                "component %s%lld: tapered guide needs >= 1 segment, its "
                "10 x nseg table (and 2 x nblocks block rows when ip[1] > "
                "0) and a positive segment length", "", (long long)k);
        return MCV_EINVAL;
      }
    }
      break;
    case MCV_OP_HSS:
    case MCV_OP_HMS: {
      int op = c.ip[0], ker = c.ip[1], rc;
      if (c.opcode == MCV_OP_HMS &&
          (c.ip[6] < 1 || c.ip[6] > MCV_MS_MAX_SCATTERED ||
           (c.ip[7] & 0xffff) > 64 || (c.ip[7] >> 16) > 64 || c.ip[7] < 0)) {
        set_msg(st, MCV_ECAPACITY,
                "component %s%lld: multiple scatterer needs 1 <= "
                "max_scattered_neutrons <= 48 and loop counts <= 64",
                "", (long long)k);
        return MCV_ECAPACITY;
      }
      bool shape_ok = c.ip[2] >= MCV_SHAPE_SPHERE && c.ip[2] <= MCV_SHAPE_BOX &&
                      op >= MCV_CSG_PRIMITIVE && op <= MCV_CSG_INTERSECTION &&
                      (op == MCV_CSG_PRIMITIVE ||
                       (c.ip[3] >= MCV_SHAPE_SPHERE && c.ip[3] <= MCV_SHAPE_BOX));
      if (!shape_ok) {
        set_msg(st, MCV_EINVAL, "component %s%lld: bad shape description", "",
                (long long)k);
        return MCV_EINVAL;
      }
      rc = validate_kernel(c, ker, k, true, st);
      if (rc) return rc;
      break;
    }
    default:
      break;
  }
  return MCV_OK;
}

bool host_is_monitor(const mcv_component& c);

int validate_chain(const mcv_chain* ch, mcv_status* st) {
  if (!ch) {
    set_msg(st, MCV_EINVAL, "chain is NULL%s", "");
    return MCV_EINVAL;
  }
  if (ch->ncomp < 1 || ch->ncomp > MCV_MAX_COMPONENTS) {
    set_msg(st, MCV_EINVAL, "chain has %s%lld components (1..32 allowed)", "",
            (long long)ch->ncomp);
    return MCV_EINVAL;
  }
  if (ch->weight_exp2 < -126 || ch->weight_exp2 > 126) {
    set_msg(st, MCV_EINVAL, "weight_exp2 %s%lld outside -126..126", "",
            (long long)ch->weight_exp2);
    return MCV_EINVAL;
  }
  int nhms = 0;
  for (int k = 0; k < ch->ncomp; ++k) {
    int rc = validate_component(ch->comp[k], k, st);
    if (rc) return rc;
    const mcv_component& c = ch->comp[k];
    nhms += c.opcode == MCV_OP_HMS;
    if ((c.opcode == MCV_OP_HSS || c.opcode == MCV_OP_HMS) &&
        c.ip[1] == MCV_KERNEL_COMPOSITE) {
      rc = validate_composite(ch, k, st);
      if (rc) return rc;
    }
  }
  if (nhms > 1) {
    set_msg(st, MCV_EINVAL, "a chain holds at most one multiple scatterer%s",
            "");
    return MCV_EINVAL;
  }
  // shared-memory tallies: monitors only, each 3 nbins doubles inside the
  // MCV_SMEM_TALLY_MAX area
  for (int k = 0; k < ch->ncomp; ++k) {
    const mcv_component& c = ch->comp[k];
    if (!(c.flags & MCV_COMP_SMEM_TALLY)) continue;
    const uint64_t m = 3 * comp_nbins(c);
    if (!host_is_monitor(c) || m == 0 || c.ip[6] < 0 ||
        (uint64_t)c.ip[6] + m > MCV_SMEM_TALLY_MAX) {
      set_msg(st, MCV_EINVAL,
              "component %s%lld: a shared-memory tally needs a monitor whose "
              "3 nbins doubles fit at ip[6] in MCV_SMEM_TALLY_MAX",
              "", (long long)k);
      return MCV_EINVAL;
    }
  }
  return MCV_OK;
}

// doubles of the regeneration kernel's shared-memory tally area: up to the
// end of the furthest MCV_COMP_SMEM_TALLY copy (validated above)
int smem_tally_words(const mcv_chain* ch) {
  int words = 0;
  for (int k = 0; k < ch->ncomp; ++k) {
    const mcv_component& c = ch->comp[k];
    if (!(c.flags & MCV_COMP_SMEM_TALLY) || !c.tally) continue;
    const int end = c.ip[6] + 3 * (int)comp_nbins(c);
    if (end > words) words = end;
  }
  return words;
}

bool has_hms(const mcv_chain* ch) {
  for (int k = 0; k < ch->ncomp; ++k)
    if (ch->comp[k].opcode == MCV_OP_HMS) return true;
  return false;
}

// Chains whose multiple scatterer runs in the warp-synchronous tree kernel
// (ms_chain_kernel): no component after it draws random numbers (the
// outputs then run the rest of the chain as they become final), and the
// launch does not ask for the thread kernel (variant 1).
bool use_ms_kernel(const mcv_chain* ch, const mcv_launch* launch) {
  if (launch && launch->variant == 1) return false;
  int k = 0;
  while (k < ch->ncomp && ch->comp[k].opcode != MCV_OP_HMS) ++k;
  if (k == ch->ncomp) return false;
  for (++k; k < ch->ncomp; ++k) {
    const int op = ch->comp[k].opcode;
    if (op == MCV_OP_HSS || op == MCV_OP_HMS || op == MCV_OP_SOURCE_SIMPLE ||
        op == MCV_OP_SNS_SOURCE)
      return false;
  }
  return true;
}

// fma: the FP64 kernel with contracted multiply-adds (launch_fp64_fma.cu)
template <typename R>
void launch_ms(mcv_ctx* ctx, const mcv_chain* chain, uint64_t ncount,
               uint64_t first, uint64_t seed, const mcv_launch* launch,
               cudaStream_t s, bool fma = false) {
  int blocks, threads;
  // one warp handles a run of incident neutrons: the grid's warps each
  // take at least 32
  launch_shape(
      ctx,
      [fma](int t) {
        return fma ? mcv_fp64_fma_ms_occupancy(t)
                   : Launchers<R>::occupancy_ms(t);
      },
      (ncount + 31) / 32 * 32, launch, &blocks, &threads);
  if (fma)
    mcv_fp64_fma_ms(blocks, threads, s, *chain, ncount, first, seed,
                    ctx->d_status);
  else
    Launchers<R>::ms(blocks, threads, s, *chain, ncount, first, seed,
                     ctx->d_status);
}

// The rarer components run in their own kernel instantiations (kX): the
// SNS source, the tapered and mesh guides, the multiple scatterer, stored
// neutrons in or out, and samples with the constant-(Q, E), E(Q), composite, SANS2D
// or DGSSXRes kernel.
bool is_exotic(const mcv_chain* ch) {
  for (int k = 0; k < ch->ncomp; ++k) {
    const int op = ch->comp[k].opcode;
    if (op == MCV_OP_HMS || op == MCV_OP_SNS_SOURCE ||
        op == MCV_OP_GUIDE_TAPERING || op == MCV_OP_NEUTRON_STORAGE ||
        op == MCV_OP_GUIDE_ANYSHAPE || op == MCV_OP_NEUTRON_TO_STORAGE)
      return true;
    if ((op == MCV_OP_HSS || op == MCV_OP_KERNEL_ELEMENT) &&
        (ch->comp[k].ip[1] == MCV_KERNEL_CONSTANT_QE ||
         ch->comp[k].ip[1] == MCV_KERNEL_E_Q ||
         ch->comp[k].ip[1] == MCV_KERNEL_COMPOSITE ||
         ch->comp[k].ip[1] == MCV_KERNEL_SANS2D ||
         ch->comp[k].ip[1] == MCV_KERNEL_DGSSXRES))
      return true;
  }
  return false;
}

int precision_ok(int precision, mcv_status* st) {
  if (precision != MCV_FP32 && precision != MCV_FP64) {
    set_msg(st, MCV_EINVAL, "precision must be 32 or 64, got %s%lld", "",
            (long long)precision);
    return 0;
  }
  return 1;
}

int launch_threads(const mcv_launch* launch) {
  int t = (launch && launch->threads_per_block > 0) ? launch->threads_per_block
                                                    : kMaxThreads;
  if (t > kMaxThreads) t = kMaxThreads;
  return (t + 31) / 32 * 32;
}

template <typename Occ>
void launch_shape(const mcv_ctx* ctx, Occ occupancy, uint64_t n,
                  const mcv_launch* launch, int* blocks, int* threads) {
  int t = launch_threads(launch);
  int per_sm = occupancy(t);
  uint64_t want = (n + t - 1) / t;
  uint64_t full = (uint64_t)ctx->sm_count * per_sm;
  uint64_t b = (launch && launch->blocks > 0) ? (uint64_t)launch->blocks
                                              : (want < full ? want : full);
  if (b < 1) b = 1;
  if (b > 0x7fffffff) b = 0x7fffffff;
  *blocks = (int)b;
  *threads = t;
}

// kX chains whose time goes into sample kernels or the multiple
// scatterer (and not into a tapered or mesh guide's loops): these run the
// kDense instantiation (FP32, Philox mode), measured faster for them and
// slower for the guide-heavy chains.
bool dense_kx_chain(const mcv_chain* ch) {
  bool samples = false;
  for (int k = 0; k < ch->ncomp; ++k) {
    const mcv_component& c = ch->comp[k];
    if (c.opcode == MCV_OP_GUIDE_TAPERING || c.opcode == MCV_OP_GUIDE_ANYSHAPE)
      return false;
    if (c.opcode == MCV_OP_HMS) samples = true;
    if (c.opcode == MCV_OP_HSS && c.ip[1] != MCV_KERNEL_ISOTROPIC &&
        c.ip[1] != MCV_KERNEL_POWDER && c.ip[1] != MCV_KERNEL_SQE_GRID)
      samples = true;
  }
  return samples;
}

template <typename R>
int launch_chain(mcv_ctx* ctx, int mode, const mcv_chain* chain,
                 uint64_t ncount, uint64_t first, uint64_t seed,
                 const float* uni, int stride, double* out_n, int* out_last,
                 const mcv_launch* launch, cudaStream_t s) {
  int blocks, threads;
  const int x = is_exotic(chain) ? (dense_kx_chain(chain) ? 2 : 1) : 0;
  launch_shape(
      ctx,
      [mode, x](int t) { return Launchers<R>::occupancy_chain(mode, x, t); },
      ncount, launch, &blocks, &threads);
  Launchers<R>::chain(mode, x, blocks, threads, s, *chain, ncount, first,
                      seed, uni, stride, out_n, out_last, ctx->d_status);
  return 0;
}

bool host_is_monitor(const mcv_component& c) {
  switch (c.opcode) {
    case MCV_OP_PSD_MONITOR:
    case MCV_OP_PSD_MONITOR_4PI:
    case MCV_OP_WAVELENGTH_MONITOR:
    case MCV_OP_POSDIV_MONITOR:
    case MCV_OP_IQE_MONITOR:
    case MCV_OP_ENERGY_MONITOR:
    case MCV_OP_THETA_TOF_4PI:
    case MCV_OP_CYL_IQE_DETECTOR:
    case MCV_OP_BANKED_DETECTOR:
      return true;
    default:
      return false;
  }
}

// The FP32 fused run uses path regeneration when asked to, or by default
// when the chain has a guide (whose bounce count varies from neutron to
// neutron) or a long segmented guide (one taking quiet blocks, ip[1] > 0:
// a neutron may die in its first segment or fly through all of them; VERDI
// 5.68e8 n/s against 5.32e8); chains without one have near-uniform paths.
bool use_regen(const mcv_chain* ch, const mcv_launch* launch) {
  if (has_hms(ch)) return false;  // the fan-out runs in the thread kernel
  if (launch && launch->variant == 1) return false;
  if (launch && (launch->variant == 2 || launch->variant == 3)) return true;
  for (int k = 0; k < ch->ncomp; ++k) {
    const mcv_component& c = ch->comp[k];
    if (c.opcode == MCV_OP_GUIDE) return true;
    if (c.opcode == MCV_OP_GUIDE_TAPERING && c.ip[1] > 0) return true;
  }
  return false;
}

// Shared memory of the regeneration kernel's tail queue for blocks of
// `threads`: one queue per warp when components follow the chain's last
// guide (variant 3 runs without it).
size_t regen_tail_bytes(const mcv_chain* ch, const mcv_launch* launch,
                        int threads) {
  if (launch && launch->variant == 3) return 0;
  int last = -1;
  for (int k = 0; k < ch->ncomp; ++k)
    if (ch->comp[k].opcode == MCV_OP_GUIDE) last = k;
  if (last < 0 || last + 1 >= ch->ncomp) return 0;
  return (size_t)(threads / 32) * kTailBytesPerWarp;
}

constexpr uint64_t kDefaultChunk = 8192;

// Layout of a staged batch: chains, then counts, then seeds.
size_t batch_bytes(int nvar) {
  return (size_t)nvar * sizeof(mcv_chain) + 2 * (size_t)nvar * sizeof(uint64_t);
}

int validate_batch(const mcv_chain* variants, int nvar, const uint64_t* counts,
                   const uint64_t* seeds, int precision, mcv_status* st) {
  if (!variants || !counts || !seeds || nvar < 1 || nvar > MCV_MAX_VARIANTS) {
    set_msg(st, MCV_EINVAL, "batched run needs 1..1024 variants%s", "");
    return MCV_EINVAL;
  }
  for (int v = 0; v < nvar; ++v) {
    int rc = validate_chain(variants + v, st);
    if (!rc && is_exotic(variants + v)) {
      set_msg(st, MCV_EINVAL,
              "batched run: no multiple scatterer, SNS source or tapered "
              "guide in a variant%s", "");
      rc = MCV_EINVAL;
    }
    if (rc) {
      if (st) st->first_bad_component = v;
      return rc;
    }
  }
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  return MCV_OK;
}

int stage_batch(void* dst, const mcv_chain* variants, int nvar,
                const uint64_t* counts, const uint64_t* seeds,
                cudaStream_t s) {
  char* d = (char*)dst;
  size_t nc = (size_t)nvar * sizeof(mcv_chain), nu = nvar * sizeof(uint64_t);
  cudaError_t e = cudaMemcpyAsync(d, variants, nc, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d + nc, counts, nu, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d + nc + nu, seeds, nu, cudaMemcpyHostToDevice, s);
  return e == cudaSuccess ? 0 : (int)e;
}

template <typename R>
void launch_batched_t(const mcv_ctx* ctx, const void* dbatch, int nvar,
                      const mcv_launch* launch, cudaStream_t s) {
  // (the kernel itself is instantiated in launch_fp32.cu / launch_fp64.cu)
  const char* d = (const char*)dbatch;
  const mcv_chain* chains = (const mcv_chain*)d;
  const uint64_t* counts = (const uint64_t*)(d + nvar * sizeof(mcv_chain));
  const uint64_t* seeds = counts + nvar;
  int t = (launch && launch->threads_per_block > 0) ? launch->threads_per_block
                                                    : kMaxThreads;
  if (t > kMaxThreads) t = kMaxThreads;
  t = (t + 31) / 32 * 32;
  size_t smem = (sizeof(mcv_chain) + 15) / 16 * 16 + 8 * (size_t)(nvar + 1);
  int per_sm = Launchers<R>::occupancy_batched(t, smem);
  int blocks = (launch && launch->blocks > 0) ? launch->blocks
                                              : ctx->sm_count * per_sm;
  uint64_t chunk = (launch && launch->chunk > 0) ? (uint64_t)launch->chunk
                                                 : kDefaultChunk;
  cudaMemsetAsync(&ctx->d_status->work_next, 0, sizeof(unsigned long long), s);
  Launchers<R>::batched(blocks, t, smem, s, chains, nvar, counts, seeds,
                        chunk, ctx->d_status);
}

void launch_batched(const mcv_ctx* ctx, const void* dbatch, int nvar,
                    int precision, const mcv_launch* launch, cudaStream_t s) {
  if (precision == MCV_FP32)
    launch_batched_t<float>(ctx, dbatch, nvar, launch, s);
  else
    launch_batched_t<double>(ctx, dbatch, nvar, launch, s);
}

uint64_t sum_counts(const uint64_t* counts, int nvar) {
  uint64_t t = 0;
  for (int v = 0; v < nvar; ++v) t += counts[v];
  return t;
}

}  // namespace

// chain validation for the other entry-point unit (noalloc.cu)
int mcv::validate_chain_for(const mcv_chain* ch, mcv_status* st) {
  int rc = validate_chain(ch, st);
  if (!rc && is_exotic(ch)) {
    set_msg(st, MCV_EINVAL,
            "batched run: no multiple scatterer, SNS source or tapered "
            "guide in a variant%s", "");
    rc = MCV_EINVAL;
  }
  return rc;
}

extern "C" {

int mcv_abi_version(void) { return MCV_ABI_VERSION; }

int mcv_struct_sizes(uint64_t* component, uint64_t* chain, uint64_t* status,
                     uint64_t* launch) {
  if (component) *component = sizeof(mcv_component);
  if (chain) *chain = sizeof(mcv_chain);
  if (status) *status = sizeof(mcv_status);
  if (launch) *launch = sizeof(mcv_launch);
  return MCV_OK;
}

int mcv_ctx_create(int device, mcv_ctx** out) {
  if (!out) return MCV_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return MCV_ENODEV;
  }
  if (device < 0 || device >= ndev) return MCV_EINVAL;
  DeviceGuard g(device);
  mcv_ctx* c = new (std::nothrow) mcv_ctx;
  if (!c) return MCV_ECAPACITY;
  c->device = device;
  c->d_batch = nullptr;
  c->batch_bytes = 0;
  c->d_grad = nullptr;
  c->grad_bytes = 0;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&c->d_status, sizeof(DevStatus)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return MCV_ECUDA;
  }
  if (cudaMemset(c->d_status, 0, sizeof(DevStatus)) != cudaSuccess) {
    cudaFree(c->d_status);
    delete c;
    return MCV_ECUDA;
  }
  *out = c;
  return MCV_OK;
}

int mcv_ctx_destroy(mcv_ctx* ctx) {
  if (!ctx) return MCV_OK;
  {
    DeviceGuard g(ctx->device);
    cudaFree(ctx->d_status);
    if (ctx->d_batch) cudaFree(ctx->d_batch);
    if (ctx->d_grad) cudaFree(ctx->d_grad);
  }
  delete ctx;
  return MCV_OK;
}

int mcv_ctx_status(mcv_ctx* ctx, void* stream, uint64_t expected,
                   mcv_status* st) {
  if (!ctx) return MCV_EINVAL;
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(st, e, "kernel execution");
  DevStatus h;
  e = cudaMemcpyAsync(&h, ctx->d_status, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_status, 0, sizeof h, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(st, e, "status read");
  int code = MCV_OK;
  if (st) {
    st->processed = h.processed;
    st->bounce_overflow = h.bounce_overflow;
    st->nonfinite = h.nonfinite;
    st->bin_oob = h.bin_oob;
    st->code = MCV_OK;
    st->message[0] = 0;
  }
  if (h.rng_overrun) {
    code = MCV_EINVAL;
    set_msg(st, code,
            "%s%lld neutrons drew more uniforms than the replay stride holds",
            "", (long long)h.rng_overrun);
  } else if (expected && h.processed != expected) {
    code = MCV_ECOUNT;
    set_msg(st, code, "processed neutron count %s%lld does not match request",
            "", (long long)h.processed);
  } else if (h.bounce_overflow) {
    code = MCV_EBOUNCE;
    set_msg(st, code, "%s%lld neutrons reached the guide bounce limit", "",
            (long long)h.bounce_overflow);
  }
  return code;
}

int mcv_run_chain(mcv_ctx* ctx, const mcv_chain* chain, uint64_t ncount,
                  uint64_t first, uint64_t seed, int precision,
                  const mcv_launch* launch, void* stream, mcv_status* st) {
  int rc = validate_chain(chain, st);
  if (rc) return rc;
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  if (!ctx) {
    set_msg(st, MCV_EINVAL, "context is NULL%s", "");
    return MCV_EINVAL;
  }
  if (ncount == 0) return st ? mcv_ctx_status(ctx, stream, 0, st) : MCV_OK;
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  if (use_ms_kernel(chain, launch)) {
    if (precision == MCV_FP32)
      launch_ms<float>(ctx, chain, ncount, first, seed, launch, s);
    else
      launch_ms<double>(ctx, chain, ncount, first, seed, launch, s,
                        launch && launch->variant == MCV_VARIANT_FP64_FMA);
  } else if (precision == MCV_FP32) {
    if (use_regen(chain, launch)) {
      int blocks, threads;
      const bool x = is_exotic(chain);
      // the kX kernels take no shared-memory tally copies
      const int tw = x ? 0 : smem_tally_words(chain);
      launch_shape(
          ctx,
          [chain, launch, x, tw](int t) {
            return Launchers<float>::occupancy_regen(
                t, (size_t)tw * 8 + regen_tail_bytes(chain, launch, t), tw,
                x);
          },
          ncount, launch, &blocks, &threads);
      Launchers<float>::regen(
          blocks, threads, (size_t)tw * 8 + regen_tail_bytes(chain, launch,
                                                             threads),
          tw, x, s, *chain, ncount, first, seed, ctx->d_status);
    } else {
      launch_chain<float>(ctx, 0, chain, ncount, first, seed, nullptr, 0,
                          nullptr, nullptr, launch, s);
    }
  } else if (launch && launch->variant == MCV_VARIANT_FP64_FMA) {
    int blocks, threads;
    const int x = is_exotic(chain) ? 1 : 0;
    launch_shape(
        ctx, [x](int t) { return mcv_fp64_fma_occupancy(x, t); }, ncount,
        launch, &blocks, &threads);
    mcv_fp64_fma_chain(x, blocks, threads, s, *chain, ncount, first, seed,
                       ctx->d_status);
  } else {
    launch_chain<double>(ctx, 0, chain, ncount, first, seed, nullptr, 0,
                         nullptr, nullptr, launch, s);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_run_chain launch");
  if (st) return mcv_ctx_status(ctx, stream, ncount, st);
  return MCV_OK;
}

int mcv_replay_uniforms(mcv_ctx* ctx, const mcv_chain* chain, uint64_t ncount,
                        uint64_t first, uint64_t seed, int precision,
                        const float* uniforms, int32_t stride,
                        double* out_neutrons, int32_t* out_last,
                        const mcv_launch* launch, void* stream,
                        mcv_status* st) {
  int rc = validate_chain(chain, st);
  if (rc) return rc;
  if (has_hms(chain)) {
    set_msg(st, MCV_EINVAL,
            "mcv_replay_uniforms: a multiple scatterer's outputs are tallied, "
            "not recorded; use mcv_run_chain%s", "");
    return MCV_EINVAL;
  }
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  if (!ctx) {
    set_msg(st, MCV_EINVAL, "context is NULL%s", "");
    return MCV_EINVAL;
  }
  if (uniforms && stride < 1) {
    set_msg(st, MCV_EINVAL, "uniform stride must be >= 1%s", "");
    return MCV_EINVAL;
  }
  if (ncount == 0) return st ? mcv_ctx_status(ctx, stream, 0, st) : MCV_OK;
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  int mode = uniforms ? 2 : 1;
  if (precision == MCV_FP32)
    launch_chain<float>(ctx, mode, chain, ncount, first, seed, uniforms,
                        stride, out_neutrons, out_last, launch, s);
  else
    launch_chain<double>(ctx, mode, chain, ncount, first, seed, uniforms,
                         stride, out_neutrons, out_last, launch, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_replay_uniforms launch");
  if (st) return mcv_ctx_status(ctx, stream, ncount, st);
  return MCV_OK;
}

int mcv_process_buffer(mcv_ctx* ctx, const mcv_chain* chain, void* neutrons,
                       uint64_t n, uint64_t first, uint64_t seed,
                       int precision, const mcv_launch* launch, void* stream,
                       mcv_status* st) {
  int rc = validate_chain(chain, st);
  if (rc) return rc;
  if (has_hms(chain)) {
    set_msg(st, MCV_EINVAL,
            "mcv_process_buffer: the multiple scatterer's fan-out needs the "
            "fused run (mcv_run_chain)%s", "");
    return MCV_EINVAL;
  }
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  if (!ctx) {
    set_msg(st, MCV_EINVAL, "context is NULL%s", "");
    return MCV_EINVAL;
  }
  if (n == 0) return st ? mcv_ctx_status(ctx, stream, 0, st) : MCV_OK;
  if (!neutrons) {
    set_msg(st, MCV_EINVAL, "neutron buffer is NULL%s", "");
    return MCV_EINVAL;
  }
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  int blocks, threads;
  const bool x = is_exotic(chain);
  if (precision == MCV_FP32) {
    launch_shape(
        ctx, [x](int t) { return Launchers<float>::occupancy_buffer(t, x); },
        n, launch, &blocks, &threads);
    Launchers<float>::buffer(blocks, threads, x, s, *chain, neutrons, n,
                             first, seed, ctx->d_status);
  } else {
    launch_shape(
        ctx, [x](int t) { return Launchers<double>::occupancy_buffer(t, x); },
        n, launch, &blocks, &threads);
    Launchers<double>::buffer(blocks, threads, x, s, *chain, neutrons, n,
                              first, seed, ctx->d_status);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_process_buffer launch");
  if (st) return mcv_ctx_status(ctx, stream, n, st);
  return MCV_OK;
}

int mcv_run_batched(mcv_ctx* ctx, const mcv_chain* variants,
                    int32_t nvariants, const uint64_t* counts,
                    const uint64_t* seeds, int precision,
                    const mcv_launch* launch, void* stream, mcv_status* st) {
  int rc = validate_batch(variants, nvariants, counts, seeds, precision, st);
  if (rc) return rc;
  if (!ctx) {
    set_msg(st, MCV_EINVAL, "context is NULL%s", "");
    return MCV_EINVAL;
  }
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  size_t need = batch_bytes(nvariants);
  if (need > ctx->batch_bytes) {
    // the previous batch may still be read by work queued on the stream
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(st, e, "mcv_run_batched");
    if (ctx->d_batch) cudaFree(ctx->d_batch);
    ctx->d_batch = nullptr;
    ctx->batch_bytes = 0;
    e = cudaMalloc(&ctx->d_batch, need);
    if (e != cudaSuccess) return cuda_fail(st, e, "mcv_run_batched staging");
    ctx->batch_bytes = need;
  }
  int e1 = stage_batch(ctx->d_batch, variants, nvariants, counts, seeds, s);
  if (e1) return cuda_fail(st, (cudaError_t)e1, "mcv_run_batched staging");
  launch_batched(ctx, ctx->d_batch, nvariants, precision, launch, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_run_batched launch");
  if (st)
    return mcv_ctx_status(ctx, stream, sum_counts(counts, nvariants), st);
  return MCV_OK;
}

int mcv_graph_create_batched(mcv_ctx* ctx, const mcv_chain* variants,
                             int32_t nvariants, const uint64_t* counts,
                             const uint64_t* seeds, int precision,
                             const mcv_launch* launch, mcv_graph** out) {
  if (!out) return MCV_EINVAL;
  *out = nullptr;
  int rc = validate_batch(variants, nvariants, counts, seeds, precision,
                          nullptr);
  if (rc) return rc;
  if (!ctx) return MCV_EINVAL;
  DeviceGuard g(ctx->device);
  mcv_graph* gr = new (std::nothrow) mcv_graph;
  if (!gr) return MCV_ECAPACITY;
  gr->ctx = ctx;
  gr->d_batch = nullptr;
  gr->graph = nullptr;
  gr->exec = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaMalloc(&gr->d_batch, batch_bytes(nvariants));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    int e1 = stage_batch(gr->d_batch, variants, nvariants, counts, seeds, s);
    e = e1 ? (cudaError_t)e1 : cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess)
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    launch_batched(ctx, gr->d_batch, nvariants, precision, launch, s);
    cudaError_t le = cudaGetLastError();
    e = cudaStreamEndCapture(s, &gr->graph);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess)
    e = cudaGraphInstantiate(&gr->exec, gr->graph, 0);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    mcv_graph_destroy(gr);
    return MCV_ECUDA;
  }
  *out = gr;
  return MCV_OK;
}

int mcv_graph_launch(mcv_graph* graph, void* stream) {
  if (!graph || !graph->exec) return MCV_EINVAL;
  DeviceGuard g(graph->ctx->device);
  cudaError_t e = cudaGraphLaunch(graph->exec, (cudaStream_t)stream);
  return e == cudaSuccess ? MCV_OK : MCV_ECUDA;
}

int mcv_graph_destroy(mcv_graph* graph) {
  if (!graph) return MCV_OK;
  {
    DeviceGuard g(graph->ctx->device);
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    if (graph->d_batch) cudaFree(graph->d_batch);
  }
  delete graph;
  return MCV_OK;
}

int mcv_backward(mcv_ctx* ctx, const mcv_chain* chain, const mcv_grad* grad,
                 uint64_t ncount, uint64_t first, uint64_t seed,
                 int precision, const mcv_launch* launch, void* stream,
                 mcv_status* st) {
  int rc = validate_chain(chain, st);
  if (rc) return rc;
  if (is_exotic(chain)) {
    set_msg(st, MCV_EINVAL,
            "mcv_backward: no gradients through the multiple scatterer, the "
            "SNS source or the tapered guide%s", "");
    return MCV_EINVAL;
  }
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  if (!grad) {
    set_msg(st, MCV_EINVAL, "gradient description is NULL%s", "");
    return MCV_EINVAL;
  }
  int hss = -1;
  for (int k = 0; k < chain->ncomp; ++k) {
    const mcv_component& c = chain->comp[k];
    if (c.opcode == MCV_OP_HSS) {
      if (hss < 0) hss = k;
      else if (grad->dparam[k] || grad->dtable[k]) {
        set_msg(st, MCV_EINVAL,
                "only the first sample is differentiated (component %s%lld)",
                "", (long long)k);
        return MCV_EINVAL;
      }
    }
    if (grad->dout[k] && !host_is_monitor(c)) {
      set_msg(st, MCV_EINVAL, "dout given for non-monitor component %s%lld",
              "", (long long)k);
      return MCV_EINVAL;
    }
  }
  if (!ctx) {
    set_msg(st, MCV_EINVAL, "context is NULL%s", "");
    return MCV_EINVAL;
  }
  if (ncount == 0) return st ? mcv_ctx_status(ctx, stream, 0, st) : MCV_OK;
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  double *px = nullptr, *py = nullptr;
  int npeaks = 0;
  if (hss >= 0 && chain->comp[hss].ip[1] == MCV_KERNEL_POWDER &&
      grad->dtable[hss]) {
    npeaks = chain->comp[hss].ip[4];
    size_t need = (2 * (size_t)npeaks + 1) * sizeof(double);
    if (need > ctx->grad_bytes) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_fail(st, e, "mcv_backward");
      if (ctx->d_grad) cudaFree(ctx->d_grad);
      ctx->d_grad = nullptr;
      ctx->grad_bytes = 0;
      e = cudaMalloc(&ctx->d_grad, need);
      if (e != cudaSuccess) return cuda_fail(st, e, "mcv_backward scratch");
      ctx->grad_bytes = need;
    }
    cudaMemsetAsync(ctx->d_grad, 0, need, s);
    px = ctx->d_grad;
    py = ctx->d_grad + npeaks + 1;
  }
  int blocks, threads;
  if (precision == MCV_FP32 && use_regen(chain, launch)) {
    // the forward's structure (regeneration, tail queue) for the replay
    auto bytes = [chain, launch](int t) {
      return regen_tail_bytes(chain, launch, t) ? (size_t)(t / 32) *
                                                      kGradTailBytesPerWarp
                                                : (size_t)0;
    };
    launch_shape(
        ctx,
        [&bytes](int t) {
          return Launchers<float>::occupancy_grad_regen(t, bytes(t));
        },
        ncount, launch, &blocks, &threads);
    size_t smem = bytes(threads);
    if (smem > 48 * 1024) {
      cudaError_t ea = Launchers<float>::allow_grad_regen_smem(smem);
      if (ea != cudaSuccess) return cuda_fail(st, ea, "mcv_backward smem");
    }
    Launchers<float>::grad_regen(blocks, threads, smem, s, *chain, *grad,
                                 ncount, first, seed, px, py,
                                 ctx->d_status);
  } else if (precision == MCV_FP32) {
    launch_shape(ctx, Launchers<float>::occupancy_grad, ncount, launch,
                 &blocks, &threads);
    Launchers<float>::grad(blocks, threads, s, *chain, *grad, ncount, first,
                           seed, px, py, ctx->d_status);
  } else {
    launch_shape(ctx, Launchers<double>::occupancy_grad, ncount, launch,
                 &blocks, &threads);
    Launchers<double>::grad(blocks, threads, s, *chain, *grad, ncount, first,
                            seed, px, py, ctx->d_status);
  }
  if (px) powder_finalize(px, py, npeaks, grad->dtable[hss], s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_backward launch");
  if (st) return mcv_ctx_status(ctx, stream, ncount, st);
  return MCV_OK;
}

int mcv_intersect(mcv_ctx* ctx, const mcv_component* hss, const double* rays,
                  uint64_t n, double* out_ts, int32_t* out_n, int precision,
                  void* stream, mcv_status* st) {
  if (!ctx || !hss || hss->opcode != MCV_OP_HSS) {
    set_msg(st, MCV_EINVAL, "mcv_intersect needs an HSS component%s", "");
    return MCV_EINVAL;
  }
  int rc = validate_component(*hss, 0, st);
  if (rc) return rc;
  if (!precision_ok(precision, st)) return MCV_EINVAL;
  if (n == 0) return MCV_OK;
  if (!rays || !out_ts || !out_n) {
    set_msg(st, MCV_EINVAL, "mcv_intersect: NULL buffer%s", "");
    return MCV_EINVAL;
  }
  DeviceGuard g(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned blocks = (unsigned)((n + 127) / 128);
  if (precision == MCV_FP32)
    Launchers<float>::intersect(blocks, 128, s, *hss, rays, n, out_ts, out_n);
  else
    Launchers<double>::intersect(blocks, 128, s, *hss, rays, n, out_ts,
                                 out_n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(st, e, "mcv_intersect launch");
  if (st) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(st, e, "mcv_intersect");
    st->code = MCV_OK;
    st->message[0] = 0;
  }
  return MCV_OK;
}

}  // extern "C"
