/*
 * ebsd_gpu.h -- C ABI of libebsdgpu.so, a GB300 (sm_103a) implementation of
 * the EBSD pattern loop of CTEMsoft's CTEMEBSD program.
 *
 * The reference is a Fortran program; its pattern loop has no library API.
 * These entry points replace, one for one, the stages of
 * ComputeEBSDPatterns (src_programs/CTEMEBSD.f90:87-672) that a Fortran
 * host would hand to the GPU through ISO_C_BINDING, and the whole program
 * (ebsd_run_namelist).  Citations are file:line in the reference tree.
 *
 * Conventions
 *   - Every int-returning call returns EBSD_OK (0) or a negative EBSD_E*
 *     code, and never exits or aborts; ebsd_last_error() gives the message.
 *   - Arrays are passed in Fortran (column-major) order, exactly as the
 *     reference declares them; nothing is transposed on the host.
 *   - Pattern pointers may be host (pageable or pinned) or device memory;
 *     the library inspects each pointer.  Device memory must be on the
 *     handle's GPU (or managed): memory of another GPU is refused with
 *     EBSD_EINVAL before any launch.  Pointers are borrowed for the
 *     duration of the call only.
 *   - One handle owns one device, one CUDA stream and its device buffers.
 *     A handle is not thread-safe; separate handles may run concurrently.
 */
#ifndef EBSD_GPU_H
#define EBSD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EBSD_OK 0
#define EBSD_EINVAL (-1)       /* bad argument or inconsistent sizes */
#define EBSD_ECUDA (-2)        /* CUDA runtime error */
#define EBSD_ENOMEM (-3)       /* device or host allocation failed */
#define EBSD_ESTATE (-4)       /* call made before its prerequisites */
#define EBSD_EIO (-5)          /* file could not be opened, read or written */
#define EBSD_EFORMAT (-6)      /* file content does not match the format */
#define EBSD_EUNSUPPORTED (-7) /* valid input outside what this build supports */
#define EBSD_ETIMEOUT (-8)     /* a bounded device-side wait gave up */

/* Scaling modes of CTEMEBSD.f90:195,630-658 (namelist scalingmode). */
#define EBSD_SCALING_NOT 0 /* 'not': full-size pattern, no binning, no gamma */
#define EBSD_SCALING_LIN 1 /* 'lin': binning only */
#define EBSD_SCALING_GAM 2 /* 'gam': binning, then pattern**gammavalue */

typedef struct ebsd_handle ebsd_handle;

/* Detector geometry: namelist EBSDdata (CTEMEBSD.f90:112-124,169-171) plus
 * the Monte-Carlo sample tilt sig read from the MC file (:344-345). */
typedef struct {
    float L;       /* scintillator distance [um] */
    float thetac;  /* detector tilt below horizontal [deg] */
    float delta;   /* pixel size on the scintillator [um] */
    int32_t numsx; /* pixels along x */
    int32_t numsy; /* pixels along y */
    float xpc;     /* pattern centre x [pixels] */
    float ypc;     /* pattern centre y [pixels] */
    double sig;    /* sample tilt from the MC file [deg] */
} ebsd_geometry;

/* What happens to each pattern after the gather (CTEMEBSD.f90:608-658). */
typedef struct {
    double prefactor;    /* :545, see ebsd_prefactor() */
    int32_t binning;     /* 1, 2, 4 or 8 (:197) */
    int32_t scalingmode; /* EBSD_SCALING_* */
    float gammavalue;    /* exponent for EBSD_SCALING_GAM */
    int32_t poisson;     /* 0: no noise; 1: Poisson noise (:611-615) */
    uint64_t seed;       /* noise seed (counter-based: results do not depend
                            on launch shape or chunking) */
} ebsd_epilogue;

/* Library version, major*10000 + minor*100 + patch. */
int ebsd_version(void);

/* Create a handle on CUDA device `device`.  Replaces the allocations of
 * CTEMEBSD.f90:394,431,477,534. */
int ebsd_create(ebsd_handle** out, int device);

/* Release every device and host resource of the handle (NULL is a no-op). */
void ebsd_destroy(ebsd_handle* h);

/* Message for the last failed call on `h`, or for the last failed
 * ebsd_create / file call on this thread when h is NULL.  Never NULL. */
const char* ebsd_last_error(const ebsd_handle* h);

/* Run the handle's work on an existing CUDA stream (cudaStream_t passed as
 * void*); NULL restores the handle's own stream. */
int ebsd_set_stream(ebsd_handle* h, void* stream);

/* Tuning and precision options (no reference counterpart; defaults keep
 * the behaviour documented here):
 *   "weights_fp64"   1 (default): the detector energy weights of
 *                    CTEMEBSD.f90:483-510 are evaluated in binary64 and
 *                    rounded once; 0: the reference's single precision.
 *                    num_el (:516) always uses the reference's arithmetic.
 *                    Takes effect at the next ebsd_set_detector.
 *   "strict_order"   0 (default): the pattern kernel sums the energy gather
 *                    of CTEMEBSD.f90:600-604 as fused dot products,
 *                    multiplies by the prefactor (:608) in binary32 and sums
 *                    binning blocks (:636) pairwise, each within a few ulps
 *                    of the reference arithmetic; 1: the reference's
 *                    summation orders, unfused, and the binary64 prefactor
 *                    multiply.
 *   "lambert_accurate" 0 (default): 1 - z as Lambert.f90:427,430 evaluate it;
 *                    1: (x^2 + y^2) / (1 + z), free of the cancellation near
 *                    the poles (cells may then differ from the reference's);
 *                    2: the pattern kernel's per-pixel geometry (rotation,
 *                    normalisation, Lambert map, cell and fractions) in
 *                    binary64 from binary64 detector directions -- the
 *                    FP64 re-evaluation of CTEMEBSD.f90:416-598 -- with the
 *                    gather in binary32: within 1e-5 of FP64 pixel by pixel
 *                    on 1001^2 masters, where a binary32 Lambert coordinate
 *                    resolves only 3e-5 of a cell; several times slower
 *                    (GB300's binary64 rate), at most 32 energy bins, no
 *                    cells diagnostic, batched jobs run as their own
 *                    launches.
 *   "l2_persist"     0 drops the persisting L2 window that ebsd_set_master
 *                    places on the master (kept by default where the device
 *                    offers one; 1 keeps it, an error if there is none).
 *   "tile_y"         pattern-kernel CTA height in pixels: 4 (default), 8, 16;
 *                    raised to 8 when the epilogue bins 8x8.
 *   "orient_per_cta" orientations per CTA, 1..64, or 0 (default): 64,
 *                    halved while the launch would have fewer than 32 CTAs
 *                    per SM.
 *   "vjp_tile_y"     tile height in pixels of ebsd_vjp and the Gauss-Newton
 *                    kernels: 4, 8, 16 or 32.  Unbinned adjoint records and
 *                    Gauss-Newton on records binned 2x2 or 4x4: 16 by
 *                    default (CTAs of 128 threads, tile_y / 4 pixel rows per
 *                    thread).  Binned adjoint records and the other
 *                    Gauss-Newton cases: 4 by default, at most 8 (one thread
 *                    per pixel); binning 8 always uses 8.
 *   "noise_index_offset"  the pattern index of the first orientation of the
 *                    next calls (default 0): Poisson noise is keyed by (seed,
 *                    pattern index, pixel), so a caller that computes a long
 *                    orientation list in pieces sets the piece's start here
 *                    and gets the noise of one call over the whole list.
 *   "vjp_orient_per_cta"  ebsd_vjp's orientations per CTA, 1..64 (default 16
 *                    for unbinned records, 8 for binned ones).
 *                    (ebsd_vjp_noalloc keeps 8 and 2, the shape its size
 *                    limit is stated for.)
 *   "gn_orient_per_cta"   the Gauss-Newton kernels', 1..64 (default 32: 3 %
 *                    faster refinement at 120x120 than 8).
 *   "host_direct"    1 (default): for a pinned host destination the pattern
 *                    kernel stores the records straight into it through its
 *                    mapped address (157 k patterns/s end to end at 640x480
 *                    on GB300, where device chunks + copies gave 87-154 k);
 *                    0: device chunks copied back on a second stream (always
 *                    the path for pageable destinations).
 *   "mc_fp32"        0 (default): ebsd_mc_run in binary64, the reference's
 *                    arithmetic; 1: the same trajectory steps in binary32,
 *                    statistically equivalent and, since GB300's binary64
 *                    units bound the default, about 16x faster (62.6 M vs
 *                    3.8 M electrons/s at the CTEMMC defaults). */
int ebsd_set_option(ebsd_handle* h, const char* key, int64_t value);

/* Master pattern upload.  sr is the host array srtmp(-npx:npx,-npy:npy,nE,
 * numset) of CTEMEBSD.f90:394-400 (Fortran order, x fastest); the atom sets
 * are summed in set order as sr = sum(srtmp,4) at :404. */
int ebsd_set_master(ebsd_handle* h, const float* sr, int32_t npx, int32_t npy, int32_t nE,
                    int32_t numset);

/* Let handle dst use the master pattern of src (same device) without a
 * copy: several detectors (each its own handle) share one device master
 * and its energy-interleaved layouts.  No reference counterpart (the
 * reference runs one detector per process). */
int ebsd_share_master(ebsd_handle* dst, const ebsd_handle* src);

/* Detector set-up: the scintillator direction cosines (CTEMEBSD.f90:416-452)
 * and the Monte-Carlo energy weights accum_e_detector (:476-510) for bins
 * Emin..Emax (1-based, inclusive, from ebsd_energy_window).  accum_e is the
 * host array accum_e(numEbins,-nsx:nsx,-nsy:nsy) (:348-349).  *num_el
 * receives nint(sum(accum_e_detector)) of :516 (may be NULL).  The master
 * must be set first (its nE must equal numEbins, :388-393). */
int ebsd_set_detector(ebsd_handle* h, const ebsd_geometry* g, const int32_t* accum_e,
                      int32_t nsx, int32_t nsy, int32_t numEbins, int32_t Emin, int32_t Emax,
                      int32_t* num_el);

/* Let handle dst use the detector of src (same device) without setting it
 * up again: the master, the MC histogram, the energy window, num_el and the
 * detector tables of CTEMEBSD.f90:416-516 are shared, not copied, so jobs
 * on one detector geometry that differ only in epilogue (binning, gamma,
 * prefactor, noise) or orientations pay for one set-up.  A handle that later
 * changes its geometry (ebsd_set_detector, or ebsd_refine of the pattern
 * centre) first takes tables of its own, so the others are unaffected;
 * the shared arrays live until the last handle holding them is destroyed.
 * dst keeps its own options and launch shape.  No reference counterpart. */
int ebsd_share_detector(ebsd_handle* dst, const ebsd_handle* src);

/* Energy window of CTEMEBSD.f90:361-367 (1-based bin indices). */
int ebsd_energy_window(float energymin, float energymax, double Ehistmin, double Ebinsize,
                       int32_t numEbins, int32_t* Emin, int32_t* Emax);

/* Intensity prefactor of CTEMEBSD.f90:545. */
double ebsd_prefactor(double beamcurrent, double dwelltime, int32_t num_el);

/* Size of one output record for epilogue e: (numsx,numsy) for 'not' or
 * binning 1, else (numsx/binning, numsy/binning) (:524-525,654-658). */
int ebsd_output_dims(const ebsd_handle* h, const ebsd_epilogue* e, int32_t* nx, int32_t* ny);

/* The pattern loop, CTEMEBSD.f90:573-658: for each of the n quaternions
 * (scalar first, n x 4 floats, quatang(4,numeuler) of :270-273) compute
 * one pattern, apply e, and write record o at out + o*nx*ny (nx*ny from
 * ebsd_output_dims, x fastest).  quats/out may each be host or device. */
int ebsd_forward(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                 float* out);

/* One job of a batch: the orientations of one detector (its handle holds
 * the detector and, possibly shared, master) with its own epilogue. */
typedef struct {
    ebsd_handle* source;    /* handle with this job's master and detector */
    const float* quats;     /* device memory, n x 4 (scalar first) */
    int64_t n;
    ebsd_epilogue epilogue; /* prefactor, binning 1/2/4/8, 'not'/'lin'/'gam' */
    float* out;             /* device memory, n records of the job's output size */
} ebsd_job;

#define EBSD_BATCH_GRAPH 1 /* capture the batch in a CUDA graph and replay it */
#define EBSD_BATCH_QUEUE_ALL 2 /* every job through the persistent queue kernel */

/* Launch-shape autotuner (no reference counterpart): times the pattern
 * kernel for this handle's detector and epilogue over n_sample orientations
 * at 128, 256 and 512 pixels per CTA x 1 to 64 orientations per CTA,
 * applies the fastest, and appends it to cache_path (a text file of
 * "shape key|tile_y|orient_per_cta|us per pattern" lines; NULL = no file).
 * A shape already in the file is applied without timing.  Any of the
 * outputs may be NULL. */
int ebsd_autotune(ebsd_handle* h, const ebsd_epilogue* e, int64_t n_sample,
                  const char* cache_path, int32_t* tile_y, int32_t* orient_per_cta,
                  float* us_per_pattern);

/* Many pattern loops of uneven size as one unit of work (no reference
 * counterpart: the reference runs one detector per process).  Jobs may
 * differ in detector size, binning, epilogue, orientation count and master
 * (phase); all sources must be on h's device.  A job whose own launch would
 * fill the GPU several times over (at least 64 CTAs per SM at its source
 * handle's launch shape, e.g. the autotuner's) runs as that launch; the
 * others share a device work queue of (job, 32 x 4, 32 x 8 or 32 x 16-pixel
 * tile at the job's tuned height, run of orientations) items consumed by a
 * persistent grid (one launch per energy-bin count, noise and tile height
 * and per 128 jobs); EBSD_BATCH_QUEUE_ALL puts every job in the queue.  With EBSD_BATCH_GRAPH all of it
 * (queue reset, launches) is captured in a CUDA graph on first use and
 * replayed for later batches with the same job list (the same buffers, sizes
 * and epilogues: new contents of the buffers are picked up).  Runs on h's
 * stream; returns when the work is queued.  Records equal those of
 * ebsd_forward on the source handles. */
int ebsd_forward_batched(ebsd_handle* h, const ebsd_job* jobs, int32_t njobs, int32_t flags);

/* Adjoint modes of ebsd_vjp. */
#define EBSD_VJP_COTANGENT 0 /* data = cotangent on the output records */
#define EBSD_VJP_NDP 1       /* data = target records; loss = 1 - normalised dot product */

/* Vector-Jacobian product of the pattern loop (no reference counterpart:
 * the reference has no derivatives; it differentiates CTEMEBSD.f90:577-608
 * and the detector set-up :416-510).  Parameters per orientation o, in
 * grad[o*6 + 0..5]: the left rotation tangent (w0, w1, w2) in radians,
 * q(w) = exp(w) (x) q with exp(w) = (cos(|w|/2), sin(|w|/2) w/|w|), and the
 * pattern centre xpc, ypc [pixels] and L [microns] (the gradient of this
 * orientation's output with respect to the detector's shared pattern
 * centre).  The forward gather is recomputed, not stored.
 *   EBSD_VJP_COTANGENT: grad = sum over record pixels of cot * dOut/dparam;
 *                       loss may be NULL.
 *   EBSD_VJP_NDP:       loss[o] = 1 - <Out,T>/(|Out||T|) against the target
 *                       record T, and grad = dloss/dparam, in one pass.
 * data holds n records of the size ebsd_output_dims gives; the epilogue
 * may bin ('lin') but not apply gamma or noise.  Pointers may be host or
 * device memory. */
int ebsd_vjp(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e, int32_t mode,
             const float* data, float* loss, float* grad);

/* ebsd_vjp for callers that cannot let the library allocate device memory
 * during the call -- hosts whose GPU memory is owned by their own pool or
 * caching allocator, and refinement loops that cannot afford the device
 * synchronisation cudaMalloc/cudaFree may cause.  It has no counterpart in
 * the reference.  Same arguments and results as ebsd_vjp, but quats, data,
 * loss (if not NULL) and grad must be device memory, and the call itself
 * allocates nothing: its per-CTA partial sums live in one fixed 8 MiB
 * device array that every GPU loading the library holds until the process
 * exits.  A detector needing more than that for a single orientation
 * (ceil(numsx/32)*ceil(numsy/8)*15 floats in EBSD_VJP_NDP mode, *6 in
 * cotangent mode) is rejected with EBSD_EUNSUPPORTED; larger batches run as
 * several launches through the array.  The first call on a device looks up
 * the array's device address (a one-time set-up), so make that first call
 * before any stream capture.  That address is kept for the life of the
 * process: after a cudaDeviceReset of the device (which also ends every
 * handle on it) this entry point must not be called again.  All calls
 * share the array: calls whose work overlaps on the GPU (other streams,
 * other threads, other handles) race and must be serialised by the caller.
 * Buffers on another GPU than the handle's are refused (EBSD_EINVAL).
 * Work is queued on the handle's stream and the call returns without
 * waiting for it. */
int ebsd_vjp_noalloc(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                     int32_t mode, const float* data, float* loss, float* grad);

/* Gauss-Newton refinement of orientations and, optionally, the detector's
 * shared pattern centre against target records (no reference counterpart).
 * The residual is the normalised-pattern difference O/|O| - T/|T|, so
 * |r|^2/2 is the loss 1 - <O,T>/(|O||T|) of ebsd_vjp.  quats, targets and
 * loss are device memory; quats are updated in place (q <- exp(dw) (x) q,
 * renormalised).  Epilogue as ebsd_vjp (binning allowed; no gamma/noise).
 *
 * Two phases per step, so callers spread over several GPUs can sum the
 * pattern-centre system across ranks in between:
 *   ebsd_gn_accumulate: per-pattern normal equations (kept in the handle)
 *     and, if pc_system != NULL, the pattern centre's Schur-complement
 *     system S dpc = r, 12 doubles (S row-major, then r), over this call's
 *     patterns; loss (may be NULL) receives each pattern's loss.
 *   ebsd_gn_apply: with dpc = NULL (orientations only) or the solved centre
 *     step, updates every orientation of the last accumulate; *max_step gets
 *     the largest rotation step in radians.
 * damping is Levenberg-Marquardt lambda relative to the diagonal. */
int ebsd_gn_accumulate(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                       const float* targets, double damping, double* pc_system, float* loss);
int ebsd_gn_apply(ebsd_handle* h, float* quats, int64_t n, double damping, const double* dpc,
                  double* max_step);

typedef struct {
    int32_t max_iterations; /* Gauss-Newton steps at most */
    int32_t refine_pc;      /* 1: also refine (xpc, ypc, L) of the shared detector */
    double damping;         /* Levenberg-Marquardt lambda, relative to the diagonal */
    double tol_rad;         /* stop when every rotation step is below this (rad) */
    double tol_pc;          /* ... and the pattern-centre step below this (px, um) */
} ebsd_gn_options;

/* The whole refinement on one GPU: ebsd_gn_accumulate / solve / apply until
 * the steps fall below the tolerances; after each centre step the detector
 * tables are rebuilt for the new geometry (the prefactor is kept: the loss
 * does not depend on it).  *geom (in/out) receives the refined detector;
 * *iterations the number of steps taken. */
int ebsd_refine(ebsd_handle* h, float* quats, int64_t n, const ebsd_epilogue* e,
                const float* targets, const ebsd_gn_options* opt, float* loss,
                ebsd_geometry* geom, int32_t* iterations);

/* ebsd_refine over several handles (one per GPU, or several on one GPU),
 * each holding a shard of the orientations: quats[k], n[k], targets[k] and
 * loss[k] (loss may be NULL, or an entry NULL) belong to handle hs[k].  All
 * handles must hold the same detector geometry.  Every iteration runs the
 * shards' accumulations concurrently (one host thread each), sums their
 * 12-number pattern-centre systems in shard order in this process, solves
 * once and applies the same centre step on every handle -- the one
 * cross-shard quantity of the refinement, reduced without any collective
 * library.  No reference counterpart. */
int ebsd_refine_sharded(ebsd_handle* const* hs, int32_t nh, float* const* quats,
                        const int64_t* n, const ebsd_epilogue* e, const float* const* targets,
                        const ebsd_gn_options* opt, float* const* loss, ebsd_geometry* geom,
                        int32_t* iterations);

/* Lambert cells of the loop (CTEMEBSD.f90:584-598) for n quaternions:
 * nix/niy (grid indices in -npx..npx) and the scaled Lambert coordinates
 * ixy0/ixy1, each [n][numsy][numsx].  Host or device pointers.  For parity
 * checking of the cell indices.  The cells are stored by the pattern kernel
 * itself (its diagnostic instantiation, at the handle's launch shape). */
int ebsd_cells(ebsd_handle* h, const float* quats, int64_t n, int32_t* nix, int32_t* niy,
               float* ixy0, float* ixy1);

/* The pattern loop (as ebsd_forward) and, from the same kernel launch, the
 * Lambert cells of every pixel and orientation (as ebsd_cells): out
 * [n][out_ny][out_nx], nix/niy/ixy0/ixy1 [n][numsy][numsx].  Device
 * pointers only (quats 16-byte aligned); no Poisson noise.  Asynchronous on
 * the handle's stream.  Reference: the loop body CTEMEBSD.f90:584-608, whose
 * cell indices (:593-598) and values (:600-608) it exposes together. */
int ebsd_forward_cells(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                       float* out, int32_t* nix, int32_t* niy, float* ixy0, float* ixy1);

/* Copy the detector weights accum_e_detector(numEbins,numsx,numsy) (zero
 * outside Emin..Emax) and direction cosines rgx/rgy/rgz(numsx,numsy) to
 * host arrays (any pointer may be NULL).  Diagnostic. */
int ebsd_get_detector(ebsd_handle* h, float* W, float* rgx, float* rgy, float* rgz);

/* ------------------------------------------------------------------ */
/* Dictionary orientation lists                                         */
/* ------------------------------------------------------------------ */

/* Cubochoric sampling of a Rodrigues fundamental zone: replaces SampleRFZ
 * (so3.f90:267-371), which fills the linked list FZlist/FZcnt.  The grid
 * has semi-edge pi^(2/3)/2 and step semi-edge/nsteps, walked x-outer,
 * z-inner from -semi-edge while below +semi-edge, the coordinate
 * accumulated by repeated addition in binary64 as the reference does;
 * each point goes cube -> ball -> Rodrigues vector in binary64 and is kept
 * if it lies in the fundamental zone of crystallographic point group pgnum
 * (1..32, International Tables order, so3.f90:59-74).  Point groups of FZ
 * type 0/1 keep the previous point's verdict for rotations of 179.999
 * degrees and more, as the reference's loop does.
 *   *count        number of members (always written);
 *   rods          count x 3 doubles, the Rodrigues vectors, or NULL;
 *   quats         count x 4 floats, the quaternions (scalar first) that
 *                 the reference's ro2qu gives (via ax2om/om2qu), ready for
 *                 ebsd_forward, or NULL.
 * At most `capacity` entries are written, in grid order; call with
 * capacity 0 to size the buffers.  Pointers are host or device memory.
 * Needs no master or detector.  nsteps 1..1000. */
int ebsd_sample_rfz(ebsd_handle* h, int32_t nsteps, int32_t pgnum, double* rods, float* quats,
                    int64_t capacity, int64_t* count);

/* ------------------------------------------------------------------ */
/* Monte-Carlo backscatter histograms (the MC file's accum_e / accum_z) */
/* ------------------------------------------------------------------ */

/* Parameters of CTEMMC's namelist MCdata (CTEMMC.f90:165-181) plus the
 * three material numbers the reference derives from the crystal file with
 * CalcDensity (:196-202); CTEMMC prints them as "Density, avZ, avA". */
typedef struct {
    double sig;       /* sample tilt about TD [deg] */
    double omega;     /* sample tilt about RD [deg] */
    double EkeV;      /* beam energy [keV] */
    double Ehistmin;  /* lowest energy bin [keV] */
    double Ebinsize;  /* energy bin width [keV] */
    double depthmax;  /* deepest exit-depth bin [nm] */
    double depthstep; /* exit-depth bin width [nm] */
    double Ze;        /* average atomic number */
    double density;   /* [g/cm^3] */
    double at_wt;     /* average atomic weight [g/mol] */
    int32_t numsx;    /* Lambert points per side, odd; nx = (numsx-1)/2 */
} ebsd_mc_params;

/* numEbins = int((EkeV-Ehistmin)/Ebinsize)+1, numzbins = int(depthmax/
 * depthstep)+1 (CTEMMC.f90:205-206); EBSD_EINVAL for inconsistent values. */
int ebsd_mc_dims(const ebsd_mc_params* p, int32_t* numEbins, int32_t* numzbins);

/* Replaces single_run (CTEMMC.f90:307-529, CSDA mode) for electrons
 * [first_electron, first_electron + n_electrons): each electron's random
 * numbers come from its own Philox4x32-10 stream keyed by `seed` (the
 * reference's sequential streams cannot be split across a GPU), mapped to
 * the reference's single-precision uniforms; results depend only on seed
 * and the electron range, so ranges run on several GPUs sum to the
 * single-GPU histogram.  Overwrites
 *   accum_e  numEbins x numsx x numsx int32, Fortran accum_e(E, x, y);
 *   accum_z  numEbins x numzbins x (2(nx/10)+1)^2 int32 (may be NULL);
 * (host or device pointers) and sets *counted (may be NULL) to the number of
 * electrons recorded in accum_e.  Exits whose energy bin or coarse depth
 * pixel would fall outside the arrays, which the reference writes past, are
 * dropped. */
int ebsd_mc_run(ebsd_handle* h, const ebsd_mc_params* p, uint64_t seed, int64_t first_electron,
                int64_t n_electrons, int32_t* accum_e, int32_t* accum_z, int64_t* counted);

/* Parsed &MCdata namelist with the defaults of CTEMMC.f90:171-183 (Ehistmin
 * defaults to 20, the reference's EkeV - 10 evaluated before the namelist is
 * read). */
typedef struct {
    char xtalname[512];
    double sig, omega;
    int32_t numsx;
    int64_t num_el;     /* electrons per thread; the run uses num_el*nthreads */
    int32_t primeseed;  /* the Philox seed here */
    double EkeV;
    char dataname[512];
    int32_t nthreads;
    double Ehistmin, Ebinsize, depthmax, depthstep;
    char MCmode[5];
    /* keys this library adds: the crystal's density [g/cm^3], average Z and
     * average atomic weight [g/mol], which the reference computes from the
     * crystal file (CalcDensity, CTEMMC.f90:196-202); reading crystal files
     * is outside this library, so they are required (default 0 = not set) */
    double density, Ze, at_wt;
} ebsd_mc_namelist;

/* Parse a namelist file (&MCdata ... / group). */
int ebsd_read_mc_namelist(const char* path, ebsd_mc_namelist* nml);

/* The whole CTEMMC program (CTEMMC.f90:48-277) for namelist file `nmlfile`
 * on device `device`: num_el*nthreads electrons, the MC file of
 * CTEMMC.f90:262-277 (the format ebsd_read_mc_file reads).  Prints the
 * reference's progress lines unless quiet != 0. */
int ebsd_run_mc_namelist(const char* nmlfile, int device, int quiet);

/* ebsd_run_mc_namelist on several GPUs: the electrons of CTEMMC.f90:307-529
 * split into ndev contiguous ranges, one per listed device and host thread,
 * each into histograms of its own, added up on the host; since every
 * electron's stream is keyed by its index in the whole run, the MC file is
 * byte for byte the single-device file.  ndev is 1..64. */
int ebsd_run_mc_namelist_devices(const char* nmlfile, const int32_t* devices, int32_t ndev,
                                 int quiet);

/* ------------------------------------------------------------------ */
/* File formats and the drop-in program                                 */
/* ------------------------------------------------------------------ */

/* The whole CTEMEBSD program (CTEMEBSD.f90:48-672) for namelist file
 * `nmlfile` (&EBSDdata, :169-205): reads the angle, MC and master files,
 * computes every pattern on device `device` and writes the unformatted
 * output file (:555-561,654-658).  Prints the reference's progress lines
 * unless quiet != 0. */
int ebsd_run_namelist(const char* nmlfile, int device, int quiet);

/* ebsd_run_namelist on several GPUs: the orientation loop of
 * CTEMEBSD.f90:573-663 is split into ndev contiguous shards, one per listed
 * device, each run by its own handle and host thread; every shard writes
 * its records at their offsets 20 + k*(4*nx*ny + 8) in the one output file,
 * which is byte for byte the single-device file.  A device listed twice
 * gets two handles sharing one device copy of the master and detector.
 * Resume (namelist key `resume`) keeps the complete records up to the
 * first incomplete one.  ndev is 1..64. */
int ebsd_run_namelist_devices(const char* nmlfile, const int32_t* devices, int32_t ndev,
                              int quiet);

/* Header of a CTEMMC output file (CTEMMC.f90:262-277). */
typedef struct {
    int32_t numEbins, numzbins, numsx, numsy;
    int64_t num_el_total;
    int32_t nthreads;
    double EkeV, Ehistmin, Ebinsize, depthmax, depthstep;
    double sig, omega;
    char MCmode[5];
} ebsd_mc_header;

/* Read an MC file (CTEMEBSD.f90:319-355).  accum_e may be NULL to read the
 * header only; otherwise it receives numEbins*numsx*numsy int32. */
int ebsd_read_mc_file(const char* path, ebsd_mc_header* hdr, int32_t* accum_e);

/* Header of a CTEMEBSDmaster output file (CTEMEBSDmaster.f90:540-568). */
typedef struct {
    int32_t npx, npy, nE, numset;
    char sqorhe[7];
} ebsd_master_header;

/* Read a master file (CTEMEBSD.f90:378-406).  EkeVs (nE floats), atomtype
 * (numset int32) and srtmp ((2npx+1)*(2npy+1)*nE*numset floats) may each
 * be NULL. */
int ebsd_read_master_file(const char* path, ebsd_master_header* hdr, float* EkeVs,
                          int32_t* atomtype, float* srtmp);

/* Parsed &EBSDdata namelist with the defaults of CTEMEBSD.f90:179-198. */
typedef struct {
    float L, thetac, delta;
    int32_t numsx, numsy;
    float xpc, ypc;
    char anglefile[512], eulerconvention[4], FZfile[512], energyfile[512], datafile[512];
    double beamcurrent, dwelltime;
    float energymin, energymax;
    int32_t binning;
    float gammavalue;
    char scalingmode[4];
    float axisangle[4];
    /* keys this library adds; defaults keep the reference's behaviour */
    int32_t poisson; /* default 1: noise on, as the reference always is */
    int64_t seed;    /* default 1 */
    int32_t resume;  /* default 0; 1: keep the complete records of an existing
                        output file with the same header and compute the rest */
    int32_t ncubochoric; /* default 0: read anglefile.  N > 0: a dictionary --
                            the orientations are the cubochoric sampling with
                            N steps per semi-edge of the fundamental zone of
                            point group pgnum (ebsd_sample_rfz), the step the
                            reference plans at CTEMEBSD.f90:292-298 */
    int32_t pgnum;       /* default 32 (m-3m); 1..32 */
} ebsd_namelist;

/* Parse a namelist file (Fortran &EBSDdata ... / group). */
int ebsd_read_namelist(const char* path, ebsd_namelist* nml);

/* Read an angle file (CTEMEBSD.f90:228-288): converts 'eu' rows (degrees;
 * 'hkl' adds 90 deg to phi1) with eu2qu and applies the optional
 * axis-angle pre-rotation.  Call with quats == NULL to get *n only. */
int ebsd_read_angle_file(const char* path, const char* eulerconvention,
                         const float axisangle[4], int64_t* n, float* quats);

/* Measured read bandwidth of one level of the memory hierarchy of a device,
 * in GB/s (best of `repeats` timed launches; CUDA events).  The
 * denominators of the pattern kernel's roofline: its gather is served by L1
 * and an L2-resident master, which a copy-based HBM figure does not bound.
 * No reference counterpart.
 *   EBSD_BW_L1:  every CTA re-reads its own 16 KB with 128-bit L1-cached loads;
 *   EBSD_BW_L2:  the grid sweeps `bytes` (e.g. 48 MB, L2-resident) with
 *                128-bit loads that bypass L1;
 *   EBSD_BW_HBM: the same sweep over `bytes` larger than L2.
 * Allocates and frees its own buffer; uses the current device's default
 * settings and changes none. */
#define EBSD_BW_L1 1
#define EBSD_BW_L2 2
#define EBSD_BW_HBM 3
int ebsd_measure_bandwidth(int32_t device, int32_t level, int64_t bytes, int32_t repeats,
                           double* gbs);

#ifdef __cplusplus
}
#endif
#endif /* EBSD_GPU_H */
