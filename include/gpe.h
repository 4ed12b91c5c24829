/*
 * gpe.h - C ABI of vaikkari_gb300, a Gross-Pitaevskii time-stepper for one
 * NVIDIA GB300 (sm_103a).
 *
 * It integrates  i d(psi)/dt = (-1/2 Lap + V + g |psi|^2) psi  on the DEC
 * discretisation of a body-centred-cubic tetrahedral mesh with the explicit
 * staggered leapfrog of the reference solver (markus-kivioja/vaikkari,
 * koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu), plus an imaginary-time
 * (ground-state) mode.  Many independent condensates ("instances") of uneven
 * sizes, couplings and traps advance together.
 *
 * Replaces, in the reference:
 *   integrateInTime(state, block_scale, minp, maxp, iteration_period, iterations)
 *       koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:218-499
 *       -> gpe_create + gpe_upload + gpe_step + gpe_download + gpe_destroy, or in
 *          one call gpe_integrate_in_time (the drop-in driver).
 *   __global__ update(next, prev, potentials, lapind, lapfacs, g, dimensions)
 *       GPUGrossPitaevskii_BCC.cu:176-216 (and its copies in the multi-GPU and
 *       MPI variants) -> the half-step inside gpe_step.
 *   getLaplacian / getPositions (GPUGrossPitaevskii_BCC.cu:69-142)
 *       -> gpe_lattice_describe.
 *   The reference reports errors by exit(EXIT_FAILURE) (helper_cuda.h
 *   checkCudaErrors, GPUGrossPitaevskii_BCC.cu:491-496); every call here
 *   returns a gpe_status instead and never exits.
 *
 * Host arrays use the reference's block order: index
 *   (((z * ny) + y) * nx + x) * slots + slot
 * for block (x, y, z) and value `slot` of that block; complex values are
 * interleaved (re, im).  The element type follows the handle's precision
 * (double for GPE_FP64, float for GPE_FP32).  GPE_FP32C exchanges the fields
 * as double (each value is split into an FP32 value and an int8 residual per
 * component on upload and recombined on download) and potential arrays as float.
 *
 * Threading: one handle per host thread; a handle owns its CUDA stream.
 */
#ifndef VAIKKARI_GB300_GPE_H
#define VAIKKARI_GB300_GPE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPE_ABI_VERSION 2

typedef enum gpe_status {
    GPE_OK = 0,
    GPE_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, enum or state           */
    GPE_ERR_CUDA = 2,             /* a CUDA runtime call failed (see gpe_last_error) */
    GPE_ERR_OUT_OF_MEMORY = 3,    /* device or pinned host allocation failed     */
    GPE_ERR_NOT_FINITE = 4,       /* NaN/Inf seen by the observables watchdog    */
    GPE_ERR_UNSUPPORTED = 5,      /* combination not built (e.g. fused TETRA12)  */
    GPE_ERR_TOO_LARGE = 6,        /* size beyond a documented maximum            */
    GPE_ERR_INTERNAL = 7,         /* lattice construction failed a self-check    */
    GPE_ERR_TIMEOUT = 8           /* a bounded wait inside a kernel ran out; the
                                     launch returned early and the fields of that
                                     step are not valid                           */
} gpe_status;

typedef enum gpe_lattice {
    /* Reference discretisation: 12 values per block at the circumcentres of the
     * BCC Delaunay tetrahedra, 4 neighbours each (GPUGrossPitaevskii_BCC.cu:69-142).
     * block_scale = the reference's block_scale; block edge = sqrt(8)*block_scale. */
    GPE_LATTICE_TETRA12 = 0,
    /* Primal-node discretisation: 2 values per block (cube corner + centre),
     * 14 Hodge-weighted edges (8 diagonal, 6 axial); block_scale = cube edge. */
    GPE_LATTICE_BCC2 = 1
} gpe_lattice;

/* GPE_FP32C: FP32 fields and arithmetic, and in real time an int8 residual per
 * component, in units of that component's ulp / 256, carried from step to step,
 * so that the accumulation of the leapfrog sums loses about 8 bits less per step
 * than FP32 storage (the stored field rounds with an exact two-sum and keeps its
 * rounding error).  BCC2, fused kernel (one-half-step and persistent variants),
 * real time; 10 instead of 8 bytes per value of a field. */
typedef enum gpe_precision { GPE_FP64 = 0, GPE_FP32 = 1, GPE_FP32C = 2 } gpe_precision;

typedef enum gpe_time_mode {
    GPE_REAL_TIME = 0,      /* staggered leapfrog, two fields (even, odd)      */
    GPE_IMAGINARY_TIME = 1  /* psi <- normalise(psi - dt H psi), one field      */
} gpe_time_mode;

typedef enum gpe_kernel_kind {
    GPE_KERNEL_AUTO = 0,   /* fused where built, plain otherwise                 */
    GPE_KERNEL_PLAIN = 1,  /* table-driven, one value per thread, any lattice    */
    GPE_KERNEL_FUSED = 2   /* shared-memory tiled, z-marching, batched: BCC2 in
                            * every storage and mode; TETRA12 in GPE_FP32, lattice
                            * or face form (real-time results equal the plain
                            * kernel's bit for bit; imaginary time fuses the sums
                            * into the step)                                     */
} gpe_kernel_kind;

typedef enum gpe_potential_kind {
    GPE_POTENTIAL_ARRAY = 0, /* V uploaded per value with gpe_upload               */
    GPE_POTENTIAL_TRAP = 1   /* V = 0.5*(trap[0] x^2 + trap[1] y^2 + trap[2] z^2),
                                evaluated in the kernel from per-axis tables       */
} gpe_potential_kind;

#define GPE_MAX_SLOTS 12
#define GPE_MAX_NEIGHBOURS 14
#define GPE_MAX_CLASSES 2

/* Stencil of a lattice, as the kernels apply it. */
typedef struct gpe_lattice_info {
    int32_t lattice;                 /* gpe_lattice                                  */
    int32_t slots;                   /* values per block                             */
    int32_t neighbours;              /* neighbours per value                         */
    int32_t classes;                 /* distinct Laplacian weights                   */
    double block_width;              /* block edge / block_scale                     */
    double cell_volume;              /* volume per value / block_scale^3             */
    double class_weight[GPE_MAX_CLASSES]; /* weight per class * block_scale^2        */
    double position[GPE_MAX_SLOTS][3];    /* value position in its block / block_scale */
    /* (dx, dy, dz, slot, class) of each neighbour, in summation order */
    int32_t entry[GPE_MAX_SLOTS][GPE_MAX_NEIGHBOURS][5];
} gpe_lattice_info;

/* The face tables of the reference's multi-GPU program, getLaplacian
 * (GPUGrossPitaevskii_BCC_multi.cu:73-271): for face f = 4 * slot + k of a
 * TETRA12 value, the neighbour's block offset (blockDirs), its slot (valueInds)
 * and the Hodge weight before scaling (hodges).  The update sums a slot's faces
 * in the reference kernel's order (perms, :314-327). */
#define GPE_FACES 48
typedef struct gpe_face_table {
    int32_t dir[GPE_FACES][3];
    int32_t slot[GPE_FACES];
    double hodge[GPE_FACES];
} gpe_face_table;

/* One condensate. */
typedef struct gpe_instance {
    int32_t nx, ny, nz;   /* blocks per axis (>= 1)                                     */
    double block_scale;   /* length unit of the lattice (see gpe_lattice)               */
    double origin[3];     /* position of the low corner of block (0,0,0)                */
    double dt;            /* time step                                                  */
    double g;             /* interaction strength                                       */
    double trap[3];       /* harmonic trap coefficients (GPE_POTENTIAL_TRAP only)       */
} gpe_instance;

typedef struct gpe_config {
    int32_t lattice;        /* gpe_lattice        */
    int32_t precision;      /* gpe_precision      */
    int32_t mode;           /* gpe_time_mode      */
    int32_t kernel;         /* gpe_kernel_kind    */
    int32_t potential;      /* gpe_potential_kind */
    int32_t num_instances;  /* >= 1               */
    const gpe_instance *instances;
    int32_t graph_steps;    /* steps per captured CUDA graph; 0 = 100, < 0 = no graphs */
    int32_t tile;           /* fused-kernel tile variant; 0 = autotuned/default.
                             * TETRA12: 0..5 = 32x4 (6 stages), 32x2 (8), 32x6 (5),
                             * 32x3 (7), 32x2 (5), 32x3 (4) block columns
                             * (gpe_variant_* describe the BCC2 variants)         */
    int32_t zchunk;         /* planes per work item of the fused kernel; 0 = auto  */
    int32_t device;         /* CUDA device ordinal                                 */
    /* TETRA12 only (the plain kernel, or the fused one in GPE_FP32).  NULL: the update of
     * GPUGrossPitaevskii_BCC.cu:213, lapfac * sum(psi_f) + (lapfac0 + V + g|psi|^2) psi.
     * Non-NULL: the Hodge (face) form of GPUGrossPitaevskii_BCC_multi.cu:329-397,
     * sum_f h_f (psi_f - psi) + (V + g|psi|^2) psi with h_f = -0.5 hodge_f / bs^2 * dt,
     * bit for bit as that kernel computes it in FP64.  The table must describe the
     * TETRA12 graph (each value's four faces) with finite weights; it is copied. */
    const gpe_face_table *faces;
} gpe_config;

/* Observables of one instance, all in FP64 (Kahan-compensated sums):
 *   norm        = sum vol |psi|^2
 *   kinetic     = sum vol Re(conj(psi) (-1/2 Lap psi))
 *   potential   = sum vol V |psi|^2
 *   interaction = sum vol g/2 |psi|^4
 *   energy      = kinetic + potential + interaction
 *   mu          = (kinetic + potential + 2 interaction) / norm                  */
typedef struct gpe_observables {
    double norm, energy, mu, kinetic, potential, interaction;
    int32_t finite; /* 0 if any sum is NaN/Inf */
    int32_t pad_;
} gpe_observables;

typedef struct gpe_handle_ *gpe_handle;

/* Version of this ABI (GPE_ABI_VERSION). */
int32_t gpe_abi_version(void);
const char *gpe_status_string(gpe_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char *gpe_last_error(void);

/* Stencil tables derived from the lattice geometry.
 * Replaces getLaplacian/getPositions, GPUGrossPitaevskii_BCC.cu:69-142. */
gpe_status gpe_lattice_describe(int32_t lattice, gpe_lattice_info *out);

/* Allocates device memory for all instances (fields zeroed).  Replaces the
 * allocation and set-up part of integrateInTime, GPUGrossPitaevskii_BCC.cu:268-405. */
gpe_status gpe_create(const gpe_config *cfg, gpe_handle *out);
gpe_status gpe_destroy(gpe_handle h);

/* Copies one instance's fields to the device.  even/odd: complex values in block
 * order; potential: V per value (unscaled; required for GPE_POTENTIAL_ARRAY,
 * ignored otherwise).  odd may be NULL in imaginary time.  Replaces the host
 * staging and cudaMemcpy3D of GPUGrossPitaevskii_BCC.cu:313-392. */
gpe_status gpe_upload(gpe_handle h, int32_t instance, const void *even, const void *odd,
                      const void *potential);
/* Copies one instance's fields back (either pointer may be NULL). */
gpe_status gpe_download(gpe_handle h, int32_t instance, void *even, void *odd);

/* The same for `count` instances in one call: every copy and layout conversion
 * is queued on the handle's stream, with one wait at the end instead of one per
 * field (each transfer has its own device staging slot; with pinned host memory
 * the copies run at the link's bandwidth).  instances[k] names the instance of
 * entry k; even/odd/potential hold one pointer per entry (odd may be NULL in
 * imaginary time, potential may be NULL for the trap form; in gpe_download_many
 * either array, or any entry, may be NULL).  No counterpart in the reference,
 * which has one condensate. */
gpe_status gpe_upload_many(gpe_handle h, int32_t count, const int32_t *instances, const void *const *even,
                           const void *const *odd, const void *const *potential);
gpe_status gpe_download_many(gpe_handle h, int32_t count, const int32_t *instances, void *const *even,
                             void *const *odd);

/* Element type of the host field arrays of gpe_upload/gpe_download and their
 * batched forms.  A GPE_FP32C handle exchanges double by default (each value
 * split into its FP32 value and int8 residuals on upload, recombined on
 * download); with GPE_FP32 it exchanges float: an upload sets the residual to
 * zero, a download rounds value + residual to float once.  That halves the host
 * link traffic for callers whose data are single precision; the residual still
 * keeps the time integration's rounding errors from accumulating.  Other
 * handles accept only their own precision.  No counterpart in the reference. */
gpe_status gpe_set_host_precision(gpe_handle h, int32_t precision);

/* Real time: advances every instance by `steps` leapfrog steps (odd <- even,
 * then even <- odd; GPUGrossPitaevskii_BCC.cu:475-481).  Imaginary time:
 * `steps` normalised Euler steps.  Asynchronous on the handle's stream. */
gpe_status gpe_step(gpe_handle h, int64_t steps);
gpe_status gpe_synchronize(gpe_handle h);

/* Observables of field 0 (even / psi) or 1 (odd) for every instance;
 * out has num_instances entries.  Returns GPE_ERR_NOT_FINITE if any is NaN/Inf. */
gpe_status gpe_observables_get(gpe_handle h, int32_t field, gpe_observables *out);

/* One round trip of every instance: upload both fields, advance `steps` steps
 * (as gpe_step), take the observables of field 0 (as gpe_observables_get) and
 * download both fields, returning when the outputs are written.  The fields and
 * observables equal those of gpe_upload_many + gpe_step + gpe_observables_get +
 * gpe_download_many.  Arrays hold num_instances pointers indexed by instance, in
 * the host element type (gpe_set_host_precision); odd_in may be NULL in
 * imaginary time; even_out, odd_out, obs and any output entry may be NULL (not
 * downloaded).  An output buffer may be any instance's input buffer.  A
 * GPE_POTENTIAL_ARRAY potential is not moved: the one last uploaded stays.
 * In real time with the fused half-step kernels (no slabs) the instances go in up
 * to four groups, contiguous in the work-item order: the copy engines move the
 * groups up and down while the SMs step the others; a group joins the running
 * step launches once its copy should have landed and leaves after its steps, and
 * the last group's download runs beside the observables.  Overlap needs
 * page-locked host buffers; a pageable one makes its copy wait for the host.
 * Replaces the reference's upload (cudaMemcpy3D, GPUGrossPitaevskii_BCC.cu:
 * 370-391), its step loop (475-481) and its download (484), which run one after
 * another. */
gpe_status gpe_round_trip(gpe_handle h, const void *const *even_in, const void *const *odd_in, int64_t steps,
                          void *const *even_out, void *const *odd_out, gpe_observables *obs);

/* Imaginary time until |mu_k - mu_{k-1}| < tol for every instance or max_steps.
 * Steps run in graph-sized chunks of G steps (gpe_config.graph_steps, 100 by
 * default).  GPE_FP64: mu comes from the reductions fused into every step and
 * the test runs on the device each step; the host polls between chunks.
 * GPE_FP32: mu of the normalised field is taken from the FP64 observables after
 * each chunk, and the test is |mu_k - mu_{k-W}| < W * tol over the last W = 10 G
 * steps (the mean change per step over that window), because the per-step
 * change of an FP32 field's mu is below the resolution of sums over FP32 values.  Outputs may be NULL; mu_out
 * receives the last mu of each instance. */
gpe_status gpe_imaginary_time(gpe_handle h, int64_t max_steps, double tol, int64_t *steps_done,
                              int32_t *converged, double *mu_out);

/* Runs gpe_step(h, steps) between two CUDA events recorded on the handle's
 * stream and returns the elapsed device time in milliseconds (the profiling
 * hook the autotuner and benchmarks use; the reference times with clock(),
 * GPUGrossPitaevskii_BCC.cu:421,488). */
gpe_status gpe_time_steps(gpe_handle h, int64_t steps, float *ms);

/* z-slab decomposition (the reference's multi-GPU strategy,
 * GPUGrossPitaevskii_BCC_multi.cu:399-917, here on one GPU): instance `upper`
 * continues instance `lower` along +z (same nx, ny and lattice; upper's origin z =
 * lower's origin z + nz * block edge).  After every half-step the library copies
 * the boundary planes of the field just written into the neighbour's padding
 * planes, so the slabs evolve exactly as one undivided grid.  Real time only. */
gpe_status gpe_link_z(gpe_handle h, int32_t lower, int32_t upper);

/* Test hook for failure detection: when plane >= 0, the fused kernel's
 * producer withholds that plane's copy in the first work item of every launch,
 * so that the consumers' bounded wait (about one second) runs out; the launch
 * returns early and the next gpe_synchronize/gpe_download/... reports
 * GPE_ERR_TIMEOUT.  plane = -1 switches it off.  No counterpart in the reference
 * (which has no device-side waits). */
gpe_status gpe_debug_inject(gpe_handle h, int32_t plane);

/* Number of fused-kernel variants (tile shape, pipeline depth, register cap)
 * that gpe_config.tile may select, and the tile shape of one of them. */
int32_t gpe_variant_count(void);
gpe_status gpe_variant_describe(int32_t variant, int32_t *tile_x, int32_t *tile_y, int32_t *stages,
                                int32_t *min_blocks);
/* Half-steps one launch of a variant advances: 1, or 2 for the variants that
 * do a whole leapfrog step per pass over HBM (BCC2, real time only; they keep a
 * second set of fields and refuse gpe_link_z).  0 for no such variant. */
int32_t gpe_variant_half_steps(int32_t variant);

/* How a variant advances time: 0 = one half-step per launch; 1 = a whole
 * leapfrog step per launch (the two-step variants above); 2 = persistent: one
 * cooperative launch per gpe_step call advances every instance by all its
 * steps, each work item starting a half-step as soon as the neighbouring items
 * it reads have finished the previous one (BCC2, real time, FP64, FP32 or
 * GPE_FP32C; refuses gpe_link_z).  -1 for no such variant.  The reference
 * launches twice per step from a host loop (GPUGrossPitaevskii_BCC.cu:475-481). */
int32_t gpe_variant_kind(int32_t variant);

/* Kernel launches the handle has issued (for accounting). */
int64_t gpe_launch_count(gpe_handle h);

/* Host buffers the handle's transfers (gpe_upload, gpe_download and their
 * batched forms) have converted in place since creation: buffers in page-locked
 * memory mapped into the handle's device's address space (cudaHostAlloc,
 * cudaHostRegister on that device), aligned to their element pair and wholly
 * inside one such allocation.  Their conversion kernels read or write the host
 * buffer over the host link directly, with no device staging or copy-engine
 * pass; every other buffer is staged.  The reference copies whole blocks with
 * cudaMemcpy3D (GPUGrossPitaevskii_BCC.cu:370-391,415,484). */
int64_t gpe_mapped_transfers(gpe_handle h);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work or record CUDA events against the library's launches. */
void *gpe_stream(gpe_handle h);

/* ---- The reference's solver call, end to end ---------------------------------
 * A vortex state file (the reference's VortexState binary format,
 * koodit/GrossPitaevskii/VortexState.cpp:49-96) and integrateInTime's own
 * set-up (GPUGrossPitaevskii_BCC.cu:222-348: grid from the domain and block_scale,
 * psi sampled at the circumcentres, potentialV3, dt from the stability bound,
 * MT19937 noise, odd field rotated by half a step) reproduced bit for bit on the
 * host, then stepped on the GPU with the TETRA12 lattice. */
typedef struct gpe_vortex_ *gpe_vortex;

typedef struct gpe_vortex_info {
    uint32_t kappa, rsize, zsize, pad_;
    double g, mu, rplug, rstep, zstep;
    double function_max;   /* searchFunctionMax (VortexState.cpp:240-248)            */
    double max_r, max_z;   /* searchMaxR/MaxZ at eps = eps_fraction * function_max    */
    double curvature;      /* integrateCurvature (:313-340)                           */
    double block_scale;    /* 2 pi / (20 sqrt(curvature)), main() :539               */
    double min_r;          /* searchMinR at the same eps (VortexState.cpp:250-257)    */
} gpe_vortex_info;

typedef struct gpe_integrate_desc {
    double block_scale;
    double minp[3], maxp[3];  /* domain, e.g. (-maxr,-maxr,-maxz) .. (maxr,maxr,maxz)      */
    double iteration_period;  /* time per iteration (1.0 in the reference)              */
    uint32_t number_of_iterations;
    uint32_t seed;            /* noise stream seed (54363 in the reference)             */
    double ratio;             /* potentialV3's RATIO (0.1 in the reference)             */
    double noise;             /* noise amplitude (0.01 in the reference)                */
    int32_t precision;        /* GPE_FP64 reproduces the reference; GPE_FP32 is faster   */
    int32_t device;
} gpe_integrate_desc;

typedef struct gpe_integrate_result {
    uint32_t xsize, ysize, zsize, steps_per_iteration;
    uint64_t values;          /* 12 * xsize * ysize * zsize                             */
    double p0[3];             /* position of block (0,0,0)                              */
    double maxpot, dt, lapfac_dt, lapfac0_dt, g_dt;
    double odd_phase[2];
    double device_ms;         /* device time of all steps (gpe_integrate_in_time)       */
    double setup_ms;          /* wall time of the set-up up to the fields on the device
                                 (gpe_integrate_in_time)                                  */
} gpe_integrate_result;

/* VortexState::load (VortexState.cpp:49-72). */
gpe_status gpe_vortex_load(const char *path, gpe_vortex *out);
void gpe_vortex_free(gpe_vortex v);
/* The diagnostics main() prints (GPUGrossPitaevskii_BCC.cu:503-548); main()
 * uses eps_fraction = 1e-5. */
gpe_status gpe_vortex_describe(gpe_vortex v, double eps_fraction, gpe_vortex_info *out);
/* VortexState::getPsi at p[3] (VortexState.cpp:204-212); out = (re, im). */
gpe_status gpe_vortex_psi(gpe_vortex v, const double *p, double *out);
/* The host set-up of integrateInTime (GPUGrossPitaevskii_BCC.cu:222-348).  Fills
 * `res`; when non-null, even/odd (complex, block order, 2*values doubles) and
 * potential (V unscaled, values doubles). */
gpe_status gpe_integrate_setup(gpe_vortex v, const gpe_integrate_desc *d, gpe_integrate_result *res,
                               double *even, double *odd, double *potential);
/* The grid integrateInTime builds for `d` (GPUGrossPitaevskii_BCC.cu:222-268):
 * xsize, ysize, zsize, values and p0 of `res`, the other fields zero.  It samples
 * nothing, so callers can size their buffers cheaply. */
gpe_status gpe_integrate_grid(const gpe_integrate_desc *d, gpe_integrate_result *res);
/* integrateInTime (GPUGrossPitaevskii_BCC.cu:218-499): set-up, then
 * number_of_iterations iterations of steps_per_iteration leapfrog steps on the
 * GPU.  The set-up's per-value work (positions, psi, V, maxpot, noise and the odd
 * phase) runs on the GPU with the values of gpe_integrate_setup, bit for bit;
 * the noise stream is drawn on the host in its order.  per_iteration (may be NULL) receives number_of_iterations+1 observables
 * of the even field, before each iteration and after the last; even_out/odd_out
 * (may be NULL) the final fields. */
gpe_status gpe_integrate_in_time(gpe_vortex v, const gpe_integrate_desc *d, gpe_integrate_result *res,
                                 gpe_observables *per_iteration, double *even_out, double *odd_out);

/* ---- The vortex relaxation (VortexState.cpp:98-185) on the GPU -----------------
 * main() (GPUGrossPitaevskii_BCC.cu:509-531) builds its vortex state by relaxing a
 * coarse profile, then a fine one resampled from it.  These calls reproduce each
 * step; gpe_vortex_relax runs iterateSolution's sweeps on the GPU. */

/* setKappa, setG and setRange with setDimensions' initial state
 * (VortexState.cpp:12-47): rsize = (rmax-rmin)/rstep rounded, zsize likewise.
 * A range that rounds to zero rows or columns is refused (the reference divides
 * by that zero and continues with NaN values). */
gpe_status gpe_vortex_create(uint32_t kappa, double g, double rmin, double rmax, double zmax, double rstep,
                             double zstep, gpe_vortex *out);
/* initialize(src) (VortexState.cpp:98-107): src's mu and its f resampled
 * (bilinear, getFunction) onto dst's grid. */
gpe_status gpe_vortex_initialize(gpe_vortex dst, gpe_vortex src);
/* VortexState::save (VortexState.cpp:74-96). */
gpe_status gpe_vortex_save(gpe_vortex v, const char *path);
/* The values f(r_i, z_j), rsize*zsize doubles row-major (row i at r_i). */
gpe_status gpe_vortex_values(gpe_vortex v, double *f);

typedef struct gpe_relax_desc {
    uint32_t maxiters;          /* iteration limit (10000 in main())                     */
    uint32_t graph_iterations;  /* iterations per CUDA graph launch; 0 = 100             */
    double eps;                 /* stop after an iteration whose diff < eps (1e-29)      */
    double ratio;               /* potentialRZ's RATIO (0.1 in the reference)           */
    int32_t device;
    int32_t pad_;
} gpe_relax_desc;

typedef struct gpe_relax_result {
    uint32_t iterations;        /* iterations run: k + 1 at the break, else maxiters   */
    uint32_t pad_;
    double diff;                /* the last iteration's diff                           */
    double mu;                  /* the state's mu afterwards                           */
    double device_ms;           /* device time of the whole call (all states)          */
} gpe_relax_result;

/* iterateSolution(potentialRZ, maxiters, eps) (VortexState.cpp:109-185) for
 * `count` independent states at once; each state's f and mu are updated in place
 * and results[k] (may be NULL) describes state k.  The sweep is the reference's
 * Gauss-Seidel order exactly; the per-iteration sums are formed per row in chunks
 * of 16 columns and over rows in groups of 16, so values agree with the
 * reference to rounding (with a CPU restatement of that order bit for bit).
 * Needs rsize >= 2.  Error
 * GPE_ERR_TIMEOUT if a sweep's bounded wait on the row above ran out. */
gpe_status gpe_vortex_relax(gpe_vortex *states, int32_t count, const gpe_relax_desc *d, gpe_relax_result *results);

/* Test hook: the relaxation sweep's division (from a correctly rounded
 * reciprocal and its low part, one Markstein correction) and __ddiv_rn on the
 * same n pairs; host
 * arrays, out ours[n] and ref[n]. */
gpe_status gpe_debug_divide(const double *a, const double *b, double *ours, double *ref, int64_t n, int32_t device);

/* ---- Field outputs (device-side downsampling) ----------------------------------
 * The reference's debug outputs, compiled out there by default
 * (GPUGrossPitaevskii_BCC.cu:18-19). */

/* Density per block over the padded block grid, (nx+2)*(ny+2)*(nz+2) uint16 in
 * x-fastest order with zero padding blocks: min(65535, trunc(unit * sum)).  With
 * reference_sum != 0 the sum is the reference's (its loop adds the first value's
 * |psi|^2 twelve times, GPUGrossPitaevskii_BCC.cu:456-459); otherwise it is the
 * block's total density.  The reference's unit is 60000 / (12 fmax^2). */
gpe_status gpe_volume_map(gpe_handle h, int32_t instance, int32_t field, double unit, int32_t reference_sum,
                          uint16_t *out);
/* One plane of blocks (padded index z_padded, value `slot`) as (nx+2)*(ny+2) RGB
 * triples: 256 * gain * (Re psi, |psi|, Im psi), below 1 -> 0, above 255 -> 255
 * (the reference draws slot 0 of plane zsize/2+1 with gain 5, :426-440). */
gpe_status gpe_slice_rgb(gpe_handle h, int32_t instance, int32_t field, int32_t z_padded, int32_t slot, double gain,
                         uint8_t *out);
/* MetaImage header <path> and data <path>.raw, as saveVolumeMap writes them
 * (GPUGrossPitaevskii_BCC.cu:38-67); spacing = block edge per axis. */
gpe_status gpe_write_metaimage(const char *path, const uint16_t *vol, uint32_t dx, uint32_t dy, uint32_t dz,
                               const double *spacing);
/* 24-bit BMP as Picture::save writes it (jukan_koodit/Output/Picture.cpp:81-129);
 * rgb = width*height triples, row 0 first. */
gpe_status gpe_write_bmp(const char *path, const uint8_t *rgb, uint32_t width, uint32_t height);

/* Observables without allocating.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc - programs whose device memory is all
 * handed out by their own pool, or latency-critical code where an allocation
 * (which may synchronise the device) is not allowed.  It needs no handle.
 *
 * field: caller-owned device memory, the condensate's complex values in block
 * order (element type by `precision`); potential: caller-owned device memory, V
 * per value (unscaled, same order and type), or NULL for the harmonic trap in
 * `inst->trap`.  Runs on `stream` (a cudaStream_t; NULL = default stream) on the
 * current device, waits for it, and fills `out` (host memory).
 *
 * Scratch memory is one array of GPE_NOALLOC_MAX_ROWS partial-sum rows held by
 * every GPU that loads the library; each row covers GPE_NOALLOC_VALUES_PER_ROW
 * values, so inputs of more than 16,777,216 values return GPE_ERR_TOO_LARGE.
 * All calls share that array: calls that overlap on a GPU race and must be
 * serialised by the caller.  No call may be made while its stream (or the
 * legacy default stream) is being captured into a graph: every call waits for
 * its stream and reads the sums back to the host, neither of which a capture
 * allows.  The array's address is looked up on a device's first call and kept
 * for the context it was found in, so after cudaDeviceReset (a new context) the
 * next call looks it up again.  It allocates nothing when it succeeds; a failure
 * records its message for gpe_last_error() as every call does.  A field that is
 * zero everywhere has no mu and returns GPE_ERR_NOT_FINITE with its own message.
 * The kinetic term uses the lattice's own weights (a face table's weights are
 * not known here). */
#define GPE_NOALLOC_MAX_ROWS 8192
#define GPE_NOALLOC_VALUES_PER_ROW 2048
gpe_status gpe_observables_noalloc(int32_t lattice, int32_t precision, const gpe_instance *inst,
                                   const void *field, const void *potential, void *stream,
                                   gpe_observables *out);

#ifdef __cplusplus
}
#endif
#endif /* VAIKKARI_GB300_GPE_H */
