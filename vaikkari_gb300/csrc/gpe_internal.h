// gpe_internal.h - host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gpe.h"
#include "gpe_device.cuh"

// An axisymmetric vortex state f(r, z) (the reference's VortexState): rsize rows
// at r = rplug + i*rstep, each of zsize values at z = j*zstep, row-major.
struct gpe_vortex_ {
    uint32_t kappa = 0, rsize = 0, zsize = 0;
    double g = 0, rplug = 0, rstep = 0, zstep = 0, mu = 0;
    std::vector<double> f;
};

namespace gpe {

// Lattice tables from the BCC geometry (gpe_lattice.cpp).
gpe_status build_lattice(gpe_lattice lattice, gpe_lattice_info *info);

// Records a message for gpe_last_error() and returns `s`.
gpe_status fail(gpe_status s, const std::string &msg);
gpe_status cuda_fail(cudaError_t e, const char *what);

// The status for an exception that reached an entry point, called inside its
// catch handler: std::bad_alloc becomes GPE_ERR_OUT_OF_MEMORY, anything else
// GPE_ERR_INTERNAL, with the entry point's name in gpe_last_error().  C callers
// cannot unwind a C++ exception, so none leaves the library.
gpe_status exception_status(const char *where) noexcept;
#define GPE_GUARD(call)                               \
    try {                                             \
        return call;                                  \
    } catch (...) {                                   \
        return ::gpe::exception_status(__func__);     \
    }

#define GPE_CUDA_TRY(expr)                                        \
    do {                                                          \
        cudaError_t gpe_e_ = (expr);                              \
        if (gpe_e_ != cudaSuccess) return ::gpe::cuda_fail(gpe_e_, #expr); \
    } while (0)

// Uploads a lattice's neighbour table to constant memory (gpe_plain.cu).
cudaError_t set_plain_table(const gpe_lattice_info &info);

// The step kernels' lattice code for a TETRA12 handle created with a face
// table (gpe_config.faces): the same layout and graph, the face-form update.
constexpr int kStepTetra12Faces = 2;

// Kernel launchers; each returns cudaGetLastError() after the launch.
struct StepLaunch {
    int lattice;          // gpe_lattice, or kStepTetra12Faces
    int precision;        // gpe_precision
    int mode;             // gpe_time_mode
    int potential;        // gpe_potential_kind
    const InstDev *inst;  // device array
    int inst_index;       // plain kernel: which instance
    int nx, ny, nz, slots;
    void *prev, *next;    // field arenas (T2*)
    const void *vpot;     // potential arena (T*) or trap tables
    const void *vbase;    // array potential: L0 + V*dt per value (T*), same index as vpot
    const ImagScalars *imag;  // imaginary time: per-instance scale of prev (device), may be null
};
cudaError_t launch_plain_step(const StepLaunch &l, cudaStream_t s);
// Planes each thread of the plain kernel marches for an instance of `values` values.
int plain_planes_per_thread(long long values, int precision);
// CTAs of the plain kernel per slot plane of an nx x ny instance.
int plain_blocks_per_plane(int nx, int ny);
// The plain step of every instance in one launch (tables from the handle).
struct PlainBatchLaunch {
    int lattice, precision, mode, potential;
    const InstDev *inst;
    const int *blk_inst, *blk_begin, *zcs;  // CTA -> instance, first CTA per instance, planes per thread
    int blocks;
    void *prev, *next;
    const void *vpot, *vbase;
    const ImagScalars *imag;
};
cudaError_t launch_plain_step_batch(const PlainBatchLaunch &l, cudaStream_t s);
// Array potential: vbase = L0 + V*dt (in the handle's precision) for one instance.
cudaError_t launch_potential_base(int precision, const InstDev *inst, int ii, int nx, int ny, int nz, int slots,
                                  const void *vpot, void *vbase, cudaStream_t s);

struct FusedLaunch {
    int precision, mode, potential, tile;
    int comp;             // real time, FP32: compensated storage (next_lo holds the residuals)
    void *next_lo;        // int8 x 2 residual per value of the next field, same padded index
    const void *lo_maps;  // CUtensorMap[num_instances][2 fields] of the residual arrays
    const void *maps;     // CUtensorMap[num_instances][2 fields][2 boxes] in device memory
    int zcmax;            // longest z-range of a work item
    int src;              // field index of prev (0 or 1)
    int *err;             // device error word (bounded-wait timeouts)
    int inject_skip_plane;  // test hook, -1 = off
    const InstDev *inst;
    const WorkItem *items;
    int num_items;
    int grid;             // CTAs
    void *prev, *next;
    const void *vpot;
    ImagScalars *imag;    // imaginary time: per-instance scalars (device), else null
    double *partials;     // imaginary time: 4 sums per work item
    unsigned int *counter;  // last-block-done counter
    const int *inst_item_begin;  // per instance id: [begin, end) item rows (2 ints each)
    int num_instances;
    double tol;
    long long step;       // host-side step index (for convergence bookkeeping)
    const long long *step_dev;  // device step counter (graphs)
    void *out_e, *out_o;  // two-step variants: the other buffer set (src = the set read)
};
cudaError_t launch_fused_step(const FusedLaunch &l, cudaStream_t s);
// The fused TETRA12 half-step (gpe_fused_t12.cu): FP32, real or imaginary time, one work
// item per CTA, a TMA ring of the previous field's planes (all 12 slots).
struct T12Launch {
    int mode, potential, variant, grid, src, inject_skip_plane;
    int face;                     // the face (Hodge) form: faces and weights from InstDev
    ImagScalars *imag;            // imaginary time: per-instance scalars
    double *partials;             // imaginary time: 4 sums per work item
    unsigned int *counter;        // imaginary time: CTAs done
    const int *inst_item_begin;   // per instance: [begin, end) item rows
    int num_instances;
    double tol;
    const InstDev *inst;
    const WorkItem *items;
    const void *maps;   // CUtensorMap[num_instances][2 fields][prev box, next box]
    const void *vmaps;  // ARRAY potential: CUtensorMap[num_instances] over L0 + V dt
    void *next;
    const void *vpot;   // TRAP: per-axis tables; ARRAY: L0 + V dt per value (face form: V dt)
    int *err;
    int tab[48];        // packed neighbour entries, slot-major
};
cudaError_t launch_t12_step(const T12Launch &l, cudaStream_t s);
int t12_variant_count();
void t12_variant(int v, int *tx, int *ty, int *stages);
// Its two 4-D maps of one field of one instance: (x, y, slot, z) over the padded
// layout; boxes = tile plus a 2-column / 1-row halo, and the interior tile, all
// 12 slots, one plane.
gpe_status make_t12_maps(void *out_map, const InstDev &d, void *field_arena, int tx, int ty);
// The map of one instance's L0 + V dt array (ARRAY potential, 4-byte values):
// box = the interior tile plus 2 columns either side (16-byte aligned), all slots.
gpe_status make_t12_vmap(void *out_map, const InstDev &d, void *vbase_arena, int tx, int ty);
// A whole leapfrog step (both half-steps) per launch: reads set l.src through
// l.maps ([instance][set][E box, O box]), writes l.out_e / l.out_o.
cudaError_t launch_twostep(const FusedLaunch &l, cudaStream_t s);
int fused_half_steps(int tile);  // 2 for the two-step variants, else 1
gpe_status make_twostep_maps(void *out_map, int precision, const InstDev &d, void *even_arena, void *odd_arena,
                             int tile);
int fused_tile_count();
void fused_tile_shape(int tile, int *tx, int *ty);
void fused_variant(int tile, int *tx, int *ty, int *stages, int *minb);
// Encodes the fused kernel's two 4-D tensor maps (halo box, interior box) of
// one field of one instance into out_map[0..1].
gpe_status make_halo_map(void *out_map, int precision, const InstDev &d, void *field_arena, int tile);
// GPE_FP32C: the 4-D map of one field's residual array (32-bit words).
gpe_status make_residual_map(void *out_map, const InstDev &d, void *lo_arena, int tile);
// Variant kinds of gpe_config.tile: one half-step per launch, a whole leapfrog
// step per launch (two-step), or the persistent kernel (many half-steps per launch).
enum VariantKind { kVariantHalfStep = 0, kVariantTwoStep = 1, kVariantPersistent = 2 };
int fused_variant_kind(int tile);
int fused_persistent_index(int tile);  // index into the persistent kernel's own variant list

// The persistent real-time kernel (gpe_persistent.cu): one cooperative launch
// advances every instance by half_steps half-steps (odd <- even first), each
// work item waiting only for its neighbouring items' epoch words.
struct PersistLaunch {
    int precision, potential, variant, comp, device;
    const InstDev *inst;
    const WorkItem *items;
    int num_items;
    const void *maps, *lo_maps;
    void *field[2];
    void *lo[2];
    const void *vpot;
    unsigned long long *ticket;
    const int *nbr_begin, *nbr;
    unsigned int *done;
    unsigned int epoch0;
    int half_steps;
    int *err;
    int inject_skip_plane;
};
cudaError_t launch_persistent(const PersistLaunch &l, cudaStream_t s, int *grid);
int persistent_variant_count();
void persistent_variant(int k, int *tx, int *ty, int *stages, int *minb);

struct ObsLaunch {
    int lattice, precision, potential;
    const InstDev *inst;
    int inst_index;
    int nx, ny, nz, slots;
    const void *field;
    const void *vpot;
    double *partials;       // 6 sums per CTA
    int max_ctas;
};
// Per-value observables partial sums for one instance; returns CTAs used.
cudaError_t launch_observables(const ObsLaunch &l, cudaStream_t s, int *ctas_used);
// CTAs the observables kernel uses for an instance of `values` values.
int observables_ctas(long long values, int max_ctas);
constexpr int kObsValuesPerBatchCta = 4096;
int observables_batch_ctas(long long values, int max_ctas);
// Observables partial rows of every instance in one launch (cta_inst: instance of
// each CTA; cta_begin: first CTA of each instance, plus the total), then one
// CTA per instance folding its rows into out[6 * i ...].
cudaError_t launch_observables_batch(int lattice, int precision, int potential, const InstDev *inst,
                                     const int *cta_inst, const int *cta_begin, int total_ctas, const void *field,
                                     const void *vpot, double *partials, cudaStream_t s);
cudaError_t launch_reduce_partials_batch(const double *partials, const int *cta_begin, int instances, double *out,
                                         cudaStream_t s);
// Reduces `ctas` partial rows (6 doubles each) in fixed order with Kahan
// compensation into out[6] (device).
cudaError_t launch_reduce_partials(const double *partials, int ctas, int width, double *out, cudaStream_t s);
// Imaginary time, plain path: from the 6 observables sums of psi_n, write
// sigma_n, mu_n and the convergence bookkeeping.
cudaError_t launch_imag_finalize_plain(const double *sums, const InstDev *inst, int inst_index,
                                       ImagScalars *imag, double tol, const long long *step_dev,
                                       cudaStream_t s);

// Layout conversion between host block order and the padded device layout.
cudaError_t launch_pack(int precision, const InstDev *inst, int inst_index, int nx, int ny, int nz,
                        int slots, const void *host_order, void *field, int is_complex, double scale,
                        cudaStream_t s);
cudaError_t launch_unpack(int precision, const InstDev *inst, int inst_index, int nx, int ny, int nz,
                          int slots, const void *field, void *host_order, const ImagScalars *imag,
                          cudaStream_t s);
// GPE_FP32C: double (or float) host order <-> FP32 field plus int8 x 2 residuals.
cudaError_t launch_pack_split(const InstDev *inst, int ii, int nx, int ny, int nz, int slots, const void *host_order,
                              void *field, void *lo, bool host_fp32, cudaStream_t s);
cudaError_t launch_unpack_join(const InstDev *inst, int ii, int nx, int ny, int nz, int slots, const void *field,
                               const void *lo, void *host_order, bool host_fp32, cudaStream_t s);
// One field of one instance in a batched transfer: its host buffer (mapped
// page-locked memory, used in place) and the first CTA of its share of the
// launch.  The array ends with a sentinel whose cta0 is the launch's CTA count.
struct XferSeg {
    const void *host;
    int inst;
    int field;
    int cta0;
    int pad;
};
constexpr int kXferValuesPerCta = 1024;  // 256 threads, 4 values each
// Every segment of a batched upload (up = true: host order -> device layout)
// or download in one launch: plain storage of `precision` (GPE_FP32, GPE_FP64),
// or comp (GPE_FP32C) with the host element float (host_fp32) or double.
cudaError_t launch_xfer_batch(int precision, bool comp, bool host_fp32, bool up, const InstDev *inst,
                              const XferSeg *segs, int nseg, int ctas, void *field0, void *field1, void *lo0, void *lo1,
                              cudaStream_t s);
// Field outputs (gpe_output.cu).
cudaError_t launch_volume(int precision, const InstDev *inst, int ii, const void *field, double unit, int quirk,
                          uint16_t *out, long long total, cudaStream_t s);
cudaError_t launch_slice(int precision, const InstDev *inst, int ii, const void *field, int kpad, int slot,
                         double gain, uint8_t *rgb, int total, cudaStream_t s);
cudaError_t launch_scale_field(int precision, const InstDev *inst, int inst_index, int nx, int ny, int nz,
                               int slots, void *field, const ImagScalars *imag, cudaStream_t s);
// Imaginary time: sigma = 1/sqrt(norm) from observables sums (no mu update).
cudaError_t launch_imag_init(const double *sums, const InstDev *inst, int inst_index, ImagScalars *imag,
                             cudaStream_t s);
cudaError_t launch_set_sigma_one(ImagScalars *imag, int n, cudaStream_t s);

// integrateInTime's set-up on the GPU (gpe_setup.cu).
struct SetupGeometry {
    uint32_t nx, ny, nz;            // blocks per axis
    uint32_t kappa, rsize, zsize;   // the vortex profile's winding and table size
    double p0[3];                   // position of block (0, 0, 0)
    double bs, W;                   // block_scale and BLOCK_WIDTH = sqrt(8)
    double bpos[12][3];             // circumcentre offsets in units of block_scale
    double ratio, coupling;         // potentialV3's RATIO and g
    double rplug, rstep, zstep;     // the profile's r origin and steps
};
// psi and V per value in block order, and the bits of max(0, max V + g|psi|^2)
// into *maxbits (which must start at 0).
cudaError_t launch_setup_sample(const SetupGeometry &geo, const double *f, double2 *psi0, double *V,
                                unsigned long long *maxbits, unsigned long long nvals, cudaStream_t s);
// even = psi (1 + amplitude * noise * 2^-31), odd = odd_phase * even and V, in
// the element type of `precision` (GPE_FP64 or GPE_FP32).
cudaError_t launch_setup_noise(int precision, const double2 *psi0, const int2 *noise, const double *V,
                               double amplitude, const double odd_phase[2], void *even, void *odd, void *pot,
                               unsigned long long nvals, cudaStream_t s);

// gpe_upload for fields and potential that are already in this handle's device
// memory, in host block order and the element type of the handle's precision
// (not GPE_FP32C).  Returns after the packing has finished.
gpe_status upload_device_fields(gpe_handle h, int32_t instance, const void *even, const void *odd,
                                const void *potential);

}  // namespace gpe
