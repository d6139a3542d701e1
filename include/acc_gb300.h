/*
 * acc_gb300.h -- C ABI of the GB300-native neutron propagation engine.
 *
 * The engine runs an instrument (a linear chain of components: source,
 * optics, sample, monitors) over N Monte-Carlo neutrons.  One neutron is the
 * ten-slot state [x, y, z, vx, vy, vz, sx, sy, t, p] (m, m/s, s, weight),
 * the layout of acc/components/sources/neutronfromstorage.py:80-81 and
 * acc/neutron.py:44-51 in mcvine/acc.
 *
 * Conventions
 *  - Plain C structs; no C++ or torch types cross this boundary.
 *  - Device buffers (tallies, tables, neutron arrays, uniforms) are owned by
 *    the caller and passed as raw device pointers.  The only memory the
 *    library allocates is a small status/work-queue block per context
 *    (mcv_ctx_create / mcv_ctx_destroy).
 *  - Every call is ordered on the caller's stream (NULL = legacy default
 *    stream).  A call given a non-NULL mcv_status synchronises that stream
 *    and fills the status; given NULL it stays asynchronous and can be
 *    captured in a CUDA graph (read the status later with mcv_ctx_status).
 *  - Every entry point returns 0 on success or an MCV_E* code, never throws,
 *    and writes a one-line reason into mcv_status.message when given one.
 *  - A context is used by one host thread at a time.
 */
#ifndef ACC_GB300_H
#define ACC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCV_ABI_VERSION 3

#define MCV_MAX_COMPONENTS 32
#define MCV_NPARAM 24
#define MCV_NIPARAM 8
#define MCV_MAX_INTERSECTIONS 10  /* acc/geometry/arrow_intersect.py:16 */
#define MCV_MAX_BOUNCES 100000    /* acc/components/optics/guide.py:17 */
#define MCV_MS_MAX_SCATTERED 48   /* output neutrons per HMS event (the
                                     reference default is 10, its UN
                                     sample uses 33) */
#define MCV_COMPOSITE_MAX 16      /* elements of a composite kernel */
#define MCV_ANYSHAPE_MAX_FACES 99 /* guide_anyshape.py:18-19, 240  */
#define MCV_ANYSHAPE_MAX_VERTICES 16
#define MCV_ANYSHAPE_MAX_BOUNCES 1000 /* guide_anyshape.py:18            */
#define MCV_EXPR_STACK 8          /* evaluation stack of an E(Q) / S(Q)
                                     program (E_Q kernel)              */
#define MCV_EXPR_MAX_OPS 256      /* instructions per E(Q) / S(Q) program */
#define MCV_SNS_E_NODES 4096      /* intervals of the SNS source's FP32
                                     inverse table of E                */
#define MCV_SNS_T_NODES 512       /* intervals of each energy row's FP32
                                     inverse table of t                */
#define MCV_SNS_TAIL_MAX 65536    /* SNS source: most FP32 tail energies */

/* ---- error codes ---------------------------------------------------- */
enum {
  MCV_OK = 0,
  MCV_EINVAL = 1,        /* bad argument or bad chain description        */
  MCV_ECUDA = 2,         /* a CUDA runtime call failed                    */
  MCV_ECOUNT = 3,        /* processed neutron count != requested          */
  MCV_EBOUNCE = 4,       /* a guide hit MCV_MAX_BOUNCES (neutron dropped) */
  MCV_ENONFINITE = 5,    /* a neutron state went NaN/Inf (dropped)        */
  MCV_EBIN = 6,          /* a tally bin index fell outside its histogram  */
  MCV_ENODEV = 7,        /* no CUDA device                                */
  MCV_ECAPACITY = 8      /* a size exceeds a documented maximum           */
};

/* ---- component opcodes ---------------------------------------------- */
enum {
  MCV_OP_ARM = 0,               /* acc/components/optics/arm.py           */
  MCV_OP_SOURCE_SIMPLE = 1,     /* acc/components/sources/source_simple.py */
  MCV_OP_GUIDE = 2,             /* acc/components/optics/guide.py          */
  MCV_OP_HSS = 3,               /* acc/components/samples/homogeneous_single_scatterer.py */
  MCV_OP_PSD_MONITOR = 4,       /* acc/components/monitors/psd_monitor.py  */
  MCV_OP_PSD_MONITOR_4PI = 5,   /* acc/components/monitors/psd_monitor_4pi.py */
  MCV_OP_WAVELENGTH_MONITOR = 6,/* acc/components/monitors/wavelength_monitor.py */
  MCV_OP_POSDIV_MONITOR = 7,    /* acc/components/monitors/posdiv_monitor.py */
  MCV_OP_IQE_MONITOR = 8,       /* acc/components/monitors/iqe_monitor.py  */
  MCV_OP_ENERGY_MONITOR = 9,    /* no reference counterpart (energy twin of the wavelength monitor) */
  MCV_OP_THETA_TOF_4PI = 10,    /* no reference counterpart (theta x tof 4pi shell) */
  MCV_OP_CYL_IQE_DETECTOR = 11, /* no reference counterpart (cylinder, binned I(Q,E)) */
  MCV_OP_BANKED_DETECTOR = 12,  /* no reference counterpart (banks x tubes x pixels x tof) */
  MCV_OP_SLIT = 13,             /* acc/components/optics/slit.py            */
  MCV_OP_BEAMSTOP = 14,         /* acc/components/optics/beamstop.py        */
  MCV_OP_HMS = 15,              /* acc/components/samples/homogeneous_multiple_scatterer.py */
  MCV_OP_GUIDE_TAPERING = 16,   /* acc/components/optics/guide_tapering.py  */
  MCV_OP_SNS_SOURCE = 17,       /* acc/components/sources/SNS_source.py     */
  MCV_OP_NEUTRON_STORAGE = 18,  /* acc/components/sources/neutronfromstorage.py */
  MCV_OP_KERNEL_ELEMENT = 19,   /* an element of a composite kernel
                                   (acc/kernels/composite.py): not run */
  MCV_OP_GUIDE_ANYSHAPE = 20,   /* acc/components/optics/guide_anyshape.py,
                                   guide_anyshape_gravity.py */
  MCV_OP_NEUTRON_TO_STORAGE = 21, /* mcvine's NeutronToStorage monitor, as
                                   acc/test/instrument_factory.py:104-113
                                   places it: saves the neutrons that reach it */
  MCV_OP_COUNT = 22
};

/* ---- shapes of the homogeneous scatterer (acc/geometry/arrow_intersect.py)
 * A shape is one primitive (A) or a binary CSG node over two primitives. */
enum {
  MCV_SHAPE_NONE = 0,
  MCV_SHAPE_SPHERE = 1,     /* dp: R                 (arrow_intersect.py:47-57)   */
  MCV_SHAPE_CYLINDER = 2,   /* dp: R, H (axis = z)   (arrow_intersect.py:59-70)   */
  MCV_SHAPE_BOX = 3         /* dp: W, H, D           (arrow_intersect.py:72-86)   */
};
enum {
  MCV_CSG_PRIMITIVE = 0,
  MCV_CSG_DIFFERENCE = 1,   /* arrow_intersect.py:88-104  */
  MCV_CSG_UNION = 2,        /* arrow_intersect.py:28-45   */
  MCV_CSG_INTERSECTION = 3  /* arrow_intersect.py:106-123 */
};

/* ---- scattering kernels (acc/kernels) -------------------------------- */
enum {
  MCV_KERNEL_ISOTROPIC = 1,   /* acc/kernels/isotropic.py:5-21, __init__.py:36-44 */
  MCV_KERNEL_POWDER = 2,      /* acc/kernels/powderdiffr.py                        */
  MCV_KERNEL_SQE_GRID = 3,    /* no reference counterpart (gridded S(Q,E) table)   */
  MCV_KERNEL_CONSTANT_QE = 4, /* acc/kernels/constant_qe.py:15-67, __init__.py:76-88 */
  MCV_KERNEL_E_Q = 5,         /* acc/kernels/E_Q.py:16-117, __init__.py:90-105     */
  MCV_KERNEL_COMPOSITE = 6,   /* acc/kernels/composite.py:7-127, __init__.py:24-34 */
  MCV_KERNEL_SANS2D = 7,      /* acc/kernels/SANS2D_ongrid.py:16-78, __init__.py:107-122 */
  MCV_KERNEL_DGSSXRES = 8     /* acc/kernels/DGSSXResKernel.py:19-98, __init__.py:124-146 */
};

/* Instructions of the postfix programs that carry the E_Q kernel's E(Q)
 * and S(Q) expressions (the reference compiles the expression strings
 * into device functions, acc/kernels/E_Q.py:16-34; here the host compiles
 * them into this form).  Each instruction is two table entries
 * {opcode, argument}.  The argument is used by CONST (the value) and POWI
 * (the integer exponent); the others ignore it. */
enum {
  MCV_EXPR_CONST = 1, MCV_EXPR_Q = 2,
  MCV_EXPR_ADD = 3, MCV_EXPR_SUB = 4, MCV_EXPR_MUL = 5, MCV_EXPR_DIV = 6,
  MCV_EXPR_POW = 7, MCV_EXPR_NEG = 8, MCV_EXPR_POWI = 9, MCV_EXPR_ATAN2 = 10,
  MCV_EXPR_MIN = 11, MCV_EXPR_MAX = 12, MCV_EXPR_MOD = 13,
  MCV_EXPR_EXP = 16, MCV_EXPR_LOG = 17, MCV_EXPR_LOG10 = 18,
  MCV_EXPR_SQRT = 19, MCV_EXPR_SIN = 20, MCV_EXPR_COS = 21, MCV_EXPR_TAN = 22,
  MCV_EXPR_ASIN = 23, MCV_EXPR_ACOS = 24, MCV_EXPR_ATAN = 25,
  MCV_EXPR_SINH = 26, MCV_EXPR_COSH = 27, MCV_EXPR_TANH = 28,
  MCV_EXPR_ASINH = 29, MCV_EXPR_ACOSH = 30, MCV_EXPR_ATANH = 31,
  MCV_EXPR_ERF = 32, MCV_EXPR_ERFC = 33, MCV_EXPR_FABS = 34,
  MCV_EXPR_FLOOR = 35, MCV_EXPR_CEIL = 36
};

/*
 * Parameter slots.  Doubles go in dp[], a float copy of the same values in
 * fp[] (the FP32 kernels read fp[], the FP64 kernels dp[]), integers in ip[].
 *
 * SOURCE_SIMPLE (source_simple.py:47-112 packs the same values)
 *   ip[0]=square ip[1]=wl_distr
 *   dp: 0 width 1 height 2 radius 3 Lambda0 4 dLambda 5 E0 6 dE 7 xw 8 yh
 *       9 dist 10 pmul
 * GUIDE (guide.py:44-50)
 *   dp: 0 ww 1 hh 2 hw1 3 hh1 4 l 5 R0 6 Qc 7 alpha 8 m 9 W
 * HSS (homogeneous_single_scatterer.py:26-102)
 *   ip[0]=csg op ip[1]=kernel ip[2]=shape A ip[3]=shape B ip[4]=npeaks / nQ
 *   ip[5]=nE
 *   dp: 0-2 shape A params, 4-6 shape B params,
 *       8 mu (absorption coefficient at 2200 m/s, 1/m), 9 sigma (1/m),
 *       POWDER: 10 unit-cell volume (A^3), 11 d_phi (deg)
 *               table: npeaks x {q_v, w_v, my_s_v2, cumulative my_s_v2}
 *               float64, q_v ascending (powderdiffr.py:112-155)
 *       SQE_GRID: 10 Qmin 11 Qmax 12 Emin 13 Emax
 *               table: nQ x nE float32 S(Q,E), row-major in Q
 *       CONSTANT_QE: 10 Q (1/A) 11 E (meV)
 *       E_Q: 10 Qmin 11 Qmax (1/A) 12 max_iter (tries of the Q draw)
 *               13: 1 when the E(Q) program does not read Q (it is then
 *               evaluated once per scatter; the results are the same)
 *               ip[4] = E(Q) instructions, ip[5] = S(Q) instructions
 *               (each 1..MCV_EXPR_MAX_OPS); table (float64) and ftable
 *               (float32): the E(Q) program then the S(Q) program,
 *               {opcode, argument} per instruction (MCV_EXPR_*)
 *       SANS2D: 10 Qx_min 11 Qx_max 12 Qy_min 13 Qy_max (1/A)
 *               ip[4] = nx, ip[5] = ny (each >= 2); table (float64) and
 *               ftable (float32): S[nx][ny], x-major (the transpose of
 *               the reference's (y, x) image)
 *       DGSSXRES: 15-17 target position (m, the sample's frame),
 *               18 target radius (m), 19 time of flight at the target
 *               (s), 20 dtof (s)
 *       COMPOSITE: ip[4] = N elements (1..MCV_COMPOSITE_MAX), in the N
 *               chain slots right after this component, each an
 *               MCV_OP_KERNEL_ELEMENT whose ip[1] is its kernel kind (not
 *               COMPOSITE), slots 8.. that kind's parameters as above and
 *               dp[22] its weight w (the weights sum to 1), dp[23] the
 *               running sum of the weights up to and including it.
 *               ip[5] bit 0: an element's scattering coefficient depends
 *               on the speed (powder), so sigma is summed per neutron;
 *               else dp[9] holds it.  dp[8] = mean of the elements' mu,
 *               dp[9] = sum of their sigma, / N when averaged.  One
 *               uniform picks element i (the first whose running sum
 *               exceeds it), which scatters, then p /= w.
 * PSD_MONITOR (psd_monitor.py:66-83)          ip: nx ny;  dp: xmin xmax ymin ymax
 * PSD_MONITOR_4PI (psd_monitor_4pi.py:56-79)  ip: nphi ntheta; dp: radius
 * WAVELENGTH_MONITOR (wavelength_monitor.py:52-74)
 *                                ip: nchan; dp: xmin xmax ymin ymax Lmin Lmax
 * POSDIV_MONITOR (posdiv_monitor.py:67-89)    ip: npos ndiv; dp: xmin xmax ymin ymax maxdiv
 * IQE_MONITOR (iqe_monitor.py:80-113)          ip: nQ nE;
 *   dp: Ei Qmin Qmax Emin Emax max_in min_in max_out min_out (degrees)
 * ENERGY_MONITOR                 ip: nchan; dp: xmin xmax ymin ymax Emin Emax
 * THETA_TOF_4PI                  ip: ntheta ntof; dp: radius tmin tmax
 *                                 (theta = polar angle from +z, 0..180 deg)
 * CYL_IQE_DETECTOR               ip: nQ nE; dp: radius height Ei Qmin Qmax Emin Emax
 * BANKED_DETECTOR                ip: nbanks ntubes npixels ntof
 *   dp: radius height bank_angle0 bank_width(rad) bank_gap(rad) tmin tmax
 * HMS (homogeneous_multiple_scatterer.py:22-342): the HSS slots, plus
 *   ip[6]=max_scattered_neutrons (1..MCV_MS_MAX_SCATTERED)
 *   ip[7]=max_ms_loops | max_ms_loops_path1 << 16
 *   dp[14]=minimum_neutron_event_probability
 *   One incident neutron gives up to max_scattered_neutrons output
 *   neutrons; the components after it run on each output in turn, drawing
 *   from the incident neutron's stream.  At most one HMS per chain;
 *   mcv_run_chain runs it (the tree kernel, or the thread kernel when a
 *   later component draws or launch variant 1 asks for it);
 *   mcv_replay_uniforms, mcv_process_buffer, mcv_backward and the batched
 *   launches reject it.
 * GUIDE_TAPERING (guide_tapering.py:22-291): nseg equal segments
 *   ip[0]=nseg  ip[1]=segments per quiet-test block (0: no blocks)
 *   dp: 0 l_seg 1 R0 2 Qcx 3 Qcy 4 alphax 5 alphay 6 mx 7 my 8 W
 *   table: float64 [10][nseg] rows w1 w2 h1 h2 ww hh whalf hhalf lwhalf
 *          lhhalf (the reference's data block, prep_inputs_kernel :122-138),
 *          then, when ip[1] > 0, [2][nblocks] rows: each block's smallest
 *          w1 or w2, and smallest h1 or h2 (nblocks = ceil(nseg / ip[1]));
 *          ftable: its float32 copy
 * SNS_SOURCE (SNS_source.py:20-207, _SNS_source_utils.py:187-223)
 *   ip: 0 square 1 nE 2 nt 3 Eidx_start 4 Eidx_stop 5 tidx_start
 *       6 tidx_stop
 *   dp: 0 xwidth 1 yheight 2 radius 3 focus_xw 4 focus_yh 5 dist 6 EPmin
 *       7 EPmax 8 prob
 *   table: float64 Es[nE] (eV), Pvec[nE], ts[nt] (us), Ptmat[nE][nt]
 *          (cumulative probabilities from the host's set-up)
 *   The FP64 kernels invert these tables per neutron (zero_find).  The
 *   FP32 kernels read ftable (float32): E_inv[MCV_SNS_E_NODES + 1] (eV at
 *   evenly spaced u, the same zero_find run on the host), Es[nE],
 *   mass[nE] (each row's probability in the t window), then
 *   t_inv[nE][MCV_SNS_T_NODES + 1] (us, evenly spaced u over each row's
 *   window), then Etail[dp 18 + dp 19] (eV): a draw u = k 2^-24 below
 *   dp 16 (u_lo: where zero_find's bracket leaves the table, or where the
 *   linear interpolation of E_inv would be coarse) takes Etail[k]
 *   (k < dp 18), one above dp 17 (u_hi) Etail[dp 18 + k - (2^24 -
 *   dp 19)], both zero_find's energies from the host; other draws outside
 *   [u_lo, u_hi] take the FP64 sampler.  dp 18 + dp 19 <=
 *   MCV_SNS_TAIL_MAX.  ftable must hold (MCV_SNS_E_NODES + 1) + 2 nE +
 *   nE (MCV_SNS_T_NODES + 1) + dp 18 + dp 19 floats: the library has no
 *   length for it and cannot check it.
 *   STS_source (STS_source.py:107-284): ip[7] bit 0 set, bit 1 = dmode;
 *   dp: 9 tanMOa 10 cylx 11 cylz 12 cylphi1 13 cylphi2 14 MRadius0
 *       15 MOffangle (rad): the face point lies on the cylindrical
 *       moderator (square ports) or on the tilted disk
 * NEUTRON_STORAGE (neutronfromstorage.py:42-82): neutron i of a run is
 *   stored neutron i mod N; table: N x 10 float64 neutrons (table_len =
 *   10 N), ftable its float32 copy
 * GUIDE_ANYSHAPE (guide_anyshape.py:96-249): a guide of flat convex
 *   mirror faces (an OFF mesh), no propagation to z = 0 first
 *   ip[0] = nfaces (1..MCV_ANYSHAPE_MAX_FACES), ip[1] = vertices a face
 *   (3..MCV_ANYSHAPE_MAX_VERTICES); dp: 0 R0 1 Qc 2 alpha 3 m 4 W
 *   table (float64) and ftable (float32): per face, 12 + 2 * nv values:
 *   centre (3), in-plane unit vectors e0, e1 (3 each), normal e2 (3),
 *   then the polygon's vertices in (e0, e1) coordinates (2 each)
 *   ip[2] bit 0: with gravity (guide_anyshape_gravity.py:25-182):
 *   dp 5-7 the gravitational acceleration in the guide's frame (m/s^2),
 *   dp 8 z_max (the mesh's largest z)
 * SLIT / BEAMSTOP (slit.py:20-108, beamstop.py:18-112)
 *                                dp: xmin xmax ymin ymax radius^2 cut
 * NEUTRON_TO_STORAGE: every neutron that reaches it is saved, unchanged
 *   and in the component's frame, into `tally`, read as 64-bit words:
 *   word 0 counts the neutrons that reached it (also past the capacity),
 *   then table_len (the capacity, >= 1) rows of 11 words: the neutron's
 *   index in the run (uint64), then x y z vx vy vz sx sy t p (float64; the
 *   FP32 kernels store p without their 2^weight_exp2 scale).  Rows are
 *   written in no fixed order; the host sorts them by index.
 *
 * Every monitor tallies into `tally`: float64 [3][n0][n1] holding
 * (N, sum p, sum p^2) per bin, the `out` array of psd_monitor.py:61-65.
 */
/* mcv_component.flags */
#define MCV_COMP_IDENTITY_ROT 1   /* rot of this hop is the identity         */
#define MCV_COMP_AGGREGATE 2      /* monitors: always warp-aggregate tally
                                     atomics (hot bins aggregate anyway) */
#define MCV_COMP_SMEM_TALLY 4     /* monitors: the FP32 path-regeneration
                                     kernel adds this monitor's entries into
                                     a per-block copy of its tally in shared
                                     memory and adds that copy to `tally`
                                     when the block ends; ip[6] = the copy's
                                     offset (doubles) in the block's tally
                                     area, which holds the 3 nbins doubles
                                     of every such monitor, at most
                                     MCV_SMEM_TALLY_MAX doubles in all (the
                                     kernels of chains with the rarer
                                     components tally it globally) */
#define MCV_SMEM_TALLY_MAX 2048

typedef struct mcv_component {
  int32_t opcode;
  int32_t flags;
  int32_t ip[MCV_NIPARAM];
  double dp[MCV_NPARAM];
  float fp[MCV_NPARAM];
  double* tally;          /* device, float64, 3*nbins, or NULL   */
  const void* table;      /* device lookup table (layout per opcode), or NULL */
  const float* ftable;    /* float32 copy of `table` for the FP32 kernels     */
  uint64_t table_len;     /* elements in table                   */
} mcv_component;

/*
 * One instrument.  rot[i], off[i] (i >= 1) take a neutron from the frame of
 * component i-1 into the frame of component i: r' = rot (r - off),
 * v' = rot v  (acc/neutron.py:18-23 with run_script.py:141-162).
 */
typedef struct mcv_chain {
  int32_t ncomp;
  int32_t flags;
  /* FP32 kernels carry every weight as p * 2^weight_exp2 (an exact power of
   * two, |weight_exp2| <= 126) and divide it out in double at tallies and
   * outputs, so that the float exponent range covers the chain's weights
   * (p0 * 2^weight_exp2 near 2^64 leaves 64 binary orders above the source
   * weight and 213 below).  FP64 kernels ignore it; 0 = no scaling. */
  int32_t weight_exp2;
  int32_t reserved;
  mcv_component comp[MCV_MAX_COMPONENTS];
  double rot[MCV_MAX_COMPONENTS][9];
  double off[MCV_MAX_COMPONENTS][3];
  float frot[MCV_MAX_COMPONENTS][9];
  float foff[MCV_MAX_COMPONENTS][3];
} mcv_chain;

/* Launch shape; zeros mean "engine default". */
typedef struct mcv_launch {
  int32_t threads_per_block;
  int32_t blocks;
  int32_t chunk;            /* neutrons per work item (batched launch) */
  int32_t variant;          /* fused FP32 kernel: 0 engine's choice,
                               1 one neutron per thread to the end of the
                               chain, 2 path regeneration (a lane whose
                               neutron leaves the chain starts the next one;
                               guides advance one bounce per step; the
                               components after the last guide run from a
                               per-warp queue in shared memory), 3 path
                               regeneration without that queue.
                               FP64 mcv_run_chain: 0 the kernel that rounds
                               every multiply and add separately (agrees
                               with the CPU restatement operation for
                               operation), MCV_VARIANT_FP64_FMA the same
                               kernel with contracted multiply-adds
                               (faster).
                               Chains with a multiple scatterer followed
                               by no source or sample run, in either
                               precision, the warp-synchronous tree kernel
                               (each lane's scattering tree as a state
                               machine, one _interactM1 call a pass on
                               all lanes); variant 1 runs them one
                               neutron per thread instead, with the same
                               results. */
} mcv_launch;

#define MCV_VARIANT_FP64_FMA 4

typedef struct mcv_status {
  int32_t code;
  int32_t first_bad_component;
  uint64_t processed;        /* neutrons that entered the chain (run_script.py:195) */
  uint64_t bounce_overflow;  /* guide loops that reached MCV_MAX_BOUNCES  */
  uint64_t nonfinite;        /* neutrons dropped for a NaN/Inf state      */
  uint64_t bin_oob;          /* tally indices out of range (skipped)      */
  char message[256];
} mcv_status;

typedef struct mcv_ctx mcv_ctx;

enum { MCV_FP32 = 32, MCV_FP64 = 64 };

/* ---- library ---------------------------------------------------------- */
int mcv_abi_version(void);
/* sizeof the ABI structs, so a binding can check its mirror. */
int mcv_struct_sizes(uint64_t* component, uint64_t* chain, uint64_t* status,
                     uint64_t* launch);

/* Context: per-device status counters and work-queue words. */
int mcv_ctx_create(int device, mcv_ctx** out);
int mcv_ctx_destroy(mcv_ctx* ctx);
/* Synchronise `stream`, read and reset the counters of the calls since the
 * last read, validate against `expected` processed neutrons (0 = skip). */
int mcv_ctx_status(mcv_ctx* ctx, void* stream, uint64_t expected,
                   mcv_status* st);

/*
 * Fused run: replaces the generated process_kernel_no_buffer of
 * acc/run_script.py:165-224 (launched from
 * acc/components/sources/SourceBase.py:36-52).  Runs neutrons with indices
 * [first, first+ncount) of the stream keyed by `seed` through the whole chain
 * in one kernel and adds into the component tallies.  Neutron i draws its
 * uniforms from Philox4x32-10 with counter (i, draw block), five 24-bit
 * uniforms per 128-bit block, so the result does not depend on the launch
 * shape, and disjoint index ranges on several devices sum to the
 * single-device run.
 */
int mcv_run_chain(mcv_ctx* ctx, const mcv_chain* chain, uint64_t ncount,
                  uint64_t first, uint64_t seed, int precision,
                  const mcv_launch* launch, void* stream, mcv_status* st);

/*
 * Replay run for parity: as mcv_run_chain, but neutron i takes its uniforms
 * from uniforms[i*stride ...] (float32, in [0,1), consumed in the draw order
 * of the reference components) instead of Philox when `uniforms` is non-NULL,
 * and writes its state when it leaves the chain into out_neutrons[i*10 ...]
 * (float64) and the index of the last component it reached into
 * out_last[i] when those are non-NULL.
 */
int mcv_replay_uniforms(mcv_ctx* ctx, const mcv_chain* chain, uint64_t ncount,
                        uint64_t first, uint64_t seed, int precision,
                        const float* uniforms, int32_t stride,
                        double* out_neutrons, int32_t* out_last,
                        const mcv_launch* launch, void* stream,
                        mcv_status* st);

/*
 * Buffered (per-component) mode: replaces ComponentBase.process /
 * call_process (acc/components/ComponentBase.py:79-129) and its stochastic
 * twin (StochasticComponentBase.py:21-54).  Applies the chain's components
 * in order to a device array neutrons[n][10] (float64 when precision is
 * MCV_FP64, float32 when MCV_FP32) in place.  A neutron whose weight is not
 * positive is left as is by later components.  Component k draws from the
 * Philox stream (seed, k+1).
 */
int mcv_process_buffer(mcv_ctx* ctx, const mcv_chain* chain, void* neutrons,
                       uint64_t n, uint64_t first, uint64_t seed,
                       int precision, const mcv_launch* launch, void* stream,
                       mcv_status* st);

/*
 * Batched run: `nvariants` instruments in one persistent launch.  No
 * counterpart in the reference, which runs one instrument per launch
 * (acc/run_script.py:210-223).  `variants`, `counts` and `seeds` are host
 * arrays; variant v runs counts[v] neutrons (indices 0..counts[v]-1 of the
 * Philox stream seeds[v]) into its own tallies.  Work items of
 * launch->chunk neutrons (0 = 8192) are handed out from the context's
 * device work counter, so variants of very different sizes balance across
 * the SMs.  The descriptions are staged in a context-owned device buffer:
 * calls sharing a context must be ordered on one stream.
 */
#define MCV_MAX_VARIANTS 1024
int mcv_run_batched(mcv_ctx* ctx, const mcv_chain* variants,
                    int32_t nvariants, const uint64_t* counts,
                    const uint64_t* seeds, int precision,
                    const mcv_launch* launch, void* stream, mcv_status* st);

/*
 * The batched launch captured once into a CUDA graph (work-counter reset +
 * kernel), replayed with mcv_graph_launch.  The graph owns device copies of
 * the variant descriptions; the variants' tallies accumulate over replays.
 * Read the counters with mcv_ctx_status after the replays.
 */
typedef struct mcv_graph mcv_graph;
int mcv_graph_create_batched(mcv_ctx* ctx, const mcv_chain* variants,
                             int32_t nvariants, const uint64_t* counts,
                             const uint64_t* seeds, int precision,
                             const mcv_launch* launch, mcv_graph** out);
int mcv_graph_launch(mcv_graph* graph, void* stream);
int mcv_graph_destroy(mcv_graph* graph);

/*
 * mcv_run_batched without any allocation.  No counterpart in the reference.
 * For callers that must not allocate device memory: a plugin inside a host
 * application that hands out every byte of device memory from its own pool,
 * or a caller that cannot take the device-wide synchronisation of freeing
 * and re-allocating a growing staging buffer.  Same arguments and results as
 * mcv_run_batched, but no context: the variant descriptions, counts, seeds,
 * counters and work-queue head live in one static device array of
 * MCV_NOALLOC_MAX_VARIANTS variants (1,034,496 bytes: 64 chain
 * descriptions of 16,144 bytes, their counts and seeds, and the counters;
 * held by every GPU that loads the library until the process exits); more
 * variants are rejected with MCV_ECAPACITY.  The first call on a device
 * looks up the array's device address, so make that first call before any
 * stream capture.  The address stays valid for the life of the device's
 * primary context: after a cudaDeviceReset in the process, do not call this
 * entry point again.  The
 * call itself zeroes the counters and the work-queue head in the array
 * before its launch; the tallies add to what they hold, as with
 * mcv_run_batched.  Every call shares the one array: calls that overlap on
 * the GPU (other streams, other host threads) race, so order them on one
 * stream.  st != NULL synchronises the stream and reads the counters back;
 * with st == NULL they are lost when the next call clears them.
 */
#define MCV_NOALLOC_MAX_VARIANTS 64
int mcv_run_batched_noalloc(const mcv_chain* variants, int32_t nvariants,
                            const uint64_t* counts, const uint64_t* seeds,
                            int precision, const mcv_launch* launch,
                            void* stream, mcv_status* st);

/*
 * Gradients of monitor tallies.  No counterpart in the reference.
 * dout[k] (monitor k, float64 per bin) is dL/d(sum p) of that monitor's
 * bins, NULL if the monitor is not in the loss.  Results are ADDED into:
 *   dparam[k], GUIDE k:  {dL/dm, dL/dalpha, dL/dW}        (first two guides)
 *   dparam[k], HSS k:    {dL/dmu_2200, dL/dsigma}  (mu at 2200 m/s, 1/m;
 *                        sigma the constant scattering coefficient, 1/m)
 *   dtable[k], HSS k:    SQE_GRID dL/dS (nQ*nE); POWDER dL/d my_s_v2
 *                        (npeaks, the per-peak constant of powderdiffr.py:129)
 * Only the first HSS of the chain is differentiated.
 */
typedef struct mcv_grad {
  const double* dout[MCV_MAX_COMPONENTS];
  double* dparam[MCV_MAX_COMPONENTS];
  double* dtable[MCV_MAX_COMPONENTS];
} mcv_grad;

/*
 * Backward run: replays neutrons [first, first+ncount) of the stream
 * `seed` -- the same neutrons, random numbers and arithmetic as
 * mcv_run_chain with the same arguments -- and accumulates the gradient of
 * L through the tallies (see mcv_grad).  Every differentiated parameter
 * enters only the neutron weight, so d(sum p)/d theta = sum p d ln p/d theta
 * over the neutrons in the bin, exact for the estimator with its random
 * numbers held fixed.  Table entries where the interpolated S is 0 receive
 * no gradient.  Tallies are not touched.
 */
int mcv_backward(mcv_ctx* ctx, const mcv_chain* chain, const mcv_grad* grad,
                 uint64_t ncount, uint64_t first, uint64_t seed,
                 int precision, const mcv_launch* launch, void* stream,
                 mcv_status* st);

/*
 * Geometry probe: the intersection times of rays with the shape of an HSS
 * component (arrow_intersect.py render + intersect).  rays[n][6] float64;
 * out_ts[n][MCV_MAX_INTERSECTIONS] float64; out_n[n] int32.
 */
int mcv_intersect(mcv_ctx* ctx, const mcv_component* hss, const double* rays,
                  uint64_t n, double* out_ts, int32_t* out_n, int precision,
                  void* stream, mcv_status* st);

#ifdef __cplusplus
}
#endif

#endif /* ACC_GB300_H */
