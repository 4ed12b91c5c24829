// gpe_api.cpp - the C ABI (include/gpe.h): handles, device arenas, uploads and
// downloads, work lists, CUDA-graph replay of step chunks, observables, and the
// imaginary-time driver.
//
// Corresponds to the host half of the reference's integrateInTime
// (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:218-499): grid sizing,
// device allocation, pre-scaling by dt (:289-307), host->device copies
// (:370-392) and the launch loop (:475-481).  Differences by design: all
// instances of a batch share one allocation and one launch per half-step, step
// chunks are replayed from captured CUDA graphs, and errors come back as status
// codes instead of exit().

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "gpe_internal.h"
#include "gpe_round_trip_plan.h"

namespace gpe {

static thread_local std::string g_last_error;

gpe_status fail(gpe_status s, const std::string &msg)
{
    g_last_error = msg;
    return s;
}

gpe_status exception_status(const char *where) noexcept
{
    gpe_status s = GPE_ERR_INTERNAL;
    const char *what = "unexpected exception";
    try {
        throw;
    } catch (const std::bad_alloc &) {
        s = GPE_ERR_OUT_OF_MEMORY;
        what = "host allocation failed";
    } catch (...) {
    }
    try {
        g_last_error = std::string(where) + ": " + what;
    } catch (...) {
    }
    return s;
}

gpe_status cuda_fail(cudaError_t e, const char *what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return GPE_ERR_OUT_OF_MEMORY;
    return GPE_ERR_CUDA;
}


}  // namespace gpe

using namespace gpe;

struct GraphKey {
    long long steps;
    int parity;
    double tol;
    int run_first, run_count;  // the work items the graph's launches cover
    bool operator<(const GraphKey &o) const
    {
        return std::tie(steps, parity, tol, run_first, run_count) <
               std::tie(o.steps, o.parity, o.tol, o.run_first, o.run_count);
    }
};

struct gpe_handle_ {
    gpe_config cfg{};
    std::vector<gpe_instance> inst;
    gpe_lattice_info lat{};
    int ns = 0;
    size_t esize = 0;  // bytes per real element on the device
    size_t hsize = 0;  // bytes per real element of a host field array (8 for GPE_FP32C unless host_fp32)
    bool host_fp32 = false;  // GPE_FP32C: host fields are float (gpe_set_host_precision)
    bool comp = false;                   // GPE_FP32C: compensated real-time storage
    void *lo[2] = {nullptr, nullptr};    // GPE_FP32C: int8 x 2 residual per value of fields 0 and 1
    std::vector<InstDev> idev_host;
    InstDev *idev = nullptr;
    size_t field_elems = 0, v_elems = 0;
    // even, odd (or psi and its ping-pong partner); the two-step variants add a
    // second set (2, 3) and alternate between the sets every step
    void *buf[4] = {nullptr, nullptr, nullptr, nullptr};
    bool two_step = false;
    void *vpot = nullptr;
    void *vbase = nullptr;  // array potential: L0 + V*dt per value for the plain kernel
    // plain kernel over a batch: CTA -> instance, first CTA per instance, planes per thread
    int *pb_inst = nullptr, *pb_begin = nullptr, *pb_zcs = nullptr;
    int pb_blocks = 0;
    bool fused = false;
    bool t12 = false;                 // the fused TETRA12 kernel (FP32, real time)
    int t12_tab[48] = {};             // its packed neighbour entries
    void *t12_vmaps = nullptr;        // its ARRAY-potential maps, one per instance
    int tile = 0, tx = 32, ty = 8, zchunk = 0, zcmax = 1;
    std::vector<WorkItem> items;
    WorkItem *items_dev = nullptr;
    int *item_begin_dev = nullptr;
    int grid = 0;
    std::vector<int> item_order;               // instances in work-item order (decreasing size)
    std::vector<int> item_first, item_count;   // per instance: its first work item and how many
    int run_first = 0, run_count = 0;          // items a real-time half-step launch covers (count 0: all)
    ImagScalars *imag = nullptr;
    double *partials = nullptr;       // fused imaginary-time rows
    unsigned int *counter = nullptr;
    void *maps = nullptr;             // fused: CUtensorMap[num_instances][2][2] (fields or buffer sets)
    void *lo_maps = nullptr;          // GPE_FP32C: CUtensorMap[num_instances][2] (residual arrays)
    int *err = nullptr;               // device error word of the bounded waits
    double *obs_partials = nullptr;   // observables CTA rows
    double *obs_sums = nullptr;       // per instance, 6 sums
    int obs_max_ctas = 2048;
    // all instances' observables in one launch: CTA -> instance, first CTA per instance
    int *obs_cta_inst = nullptr, *obs_cta_begin = nullptr;
    double *obs_batch_partials = nullptr;
    int obs_total_ctas = 0;
    void *staging = nullptr;
    size_t staging_bytes = 0;
    void *batch_staging = nullptr;  // gpe_upload_many / gpe_download_many: one slot per transfer
    size_t batch_bytes = 0;
    cudaStream_t copy_stream = nullptr;     // their host<->device copies, beside the conversions
    cudaStream_t down_stream = nullptr;     // gpe_round_trip: device->host copies beside the uploads
    std::vector<cudaEvent_t> xfer_events;   // one per transfer slot
    XferSeg *xfer_segs = nullptr;           // batched in-place transfers: the launch's segments
    size_t xfer_segs_cap = 0;
    std::vector<XferSeg> xfer_segs_host;
    cudaStream_t stream = nullptr;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    int parity = 0;      // imaginary time: which buffer holds psi; two-step: which set holds the fields
    int inject = -1;     // test hook for the bounded waits (gpe_debug_inject)
    std::vector<std::pair<int, int>> zlinks;  // (lower, upper): upper continues lower along +z
    uint32_t slots_from_above = 0, slots_from_below = 0;  // slots the stencil reads at z+1 / z-1
    bool imag_ready = false;
    bool faces = false;  // TETRA12 stepped in the face form (gpe_config.faces)
    // persistent variants: one launch per gpe_step call; per work item its
    // neighbouring items (CSR) and an epoch word, the half-steps it has completed
    bool persistent = false;
    int *nbr_begin_dev = nullptr, *nbr_dev = nullptr;
    unsigned int *done = nullptr;
    unsigned long long *ticket = nullptr;  // the persistent launch's work counter, zeroed before each launch
    unsigned int epoch = 0;      // done[] of every item after the launches queued so far
    bool epoch_reset = false;    // a launch timed out: zero done[] before the next one
    double tol = 0.0;
    long long launches = 0;
    long long mapped_transfers = 0;  // host buffers converted in place (mapped page-locked memory)
};

namespace {

size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

// The buffer that holds field f (0 even / psi, 1 odd / its partner) now.
void *field_buf(const gpe_handle_ *h, int f)
{
    if (h->cfg.mode == GPE_IMAGINARY_TIME) return h->buf[f == 0 ? h->parity : 1 - h->parity];
    return h->buf[(h->two_step ? 2 * h->parity : 0) + f];
}

// Summation order of a value's four faces in the face form: position k of slot
// s takes face 4 s + kFacePerm[s][k] of the caller's table.  This is the order
// of the reference's multi-GPU kernel (perms, GPUGrossPitaevskii_BCC_multi.cu:
// 314-327), so that the FP64 sums round as its do.
const int kFacePerm[12][4] = {{3, 2, 0, 1}, {2, 0, 1, 3}, {1, 0, 2, 3}, {1, 0, 2, 3}, {2, 0, 1, 3}, {3, 1, 0, 2},
                              {0, 1, 2, 3}, {0, 1, 2, 3}, {3, 1, 0, 2}, {2, 3, 0, 1}, {2, 3, 0, 1}, {3, 2, 0, 1}};

// A face table must describe the TETRA12 graph: the four faces of each slot are
// its four lattice neighbours in some order, each with a finite weight.
gpe_status check_face_table(const gpe_face_table &t)
{
    gpe_lattice_info lat;
    gpe_status st = build_lattice(GPE_LATTICE_TETRA12, &lat);
    if (st != GPE_OK) return fail(st, "gpe_create: lattice construction failed its self-check");
    for (int s = 0; s < 12; s++) {
        bool used[4] = {false, false, false, false};
        for (int k = 0; k < 4; k++) {
            const int f = 4 * s + k;
            if (!std::isfinite(t.hodge[f]))
                return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: face " + std::to_string(f) + " has a non-finite weight");
            int match = -1;
            for (int j = 0; j < 4 && match < 0; j++)
                if (!used[j] && lat.entry[s][j][0] == t.dir[f][0] && lat.entry[s][j][1] == t.dir[f][1] &&
                    lat.entry[s][j][2] == t.dir[f][2] && lat.entry[s][j][3] == t.slot[f])
                    match = j;
            if (match < 0)
                return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: face " + std::to_string(f) +
                                                          " is not a TETRA12 neighbour of slot " + std::to_string(s));
            used[match] = true;
        }
    }
    return GPE_OK;
}

// The lattice code the step kernels run.
int step_lattice(const gpe_handle_ *h) { return h->faces ? kStepTetra12Faces : h->cfg.lattice; }

gpe_status check_handle(gpe_handle h)
{
    if (!h) return fail(GPE_ERR_INVALID_ARGUMENT, "null handle");
    return GPE_OK;
}

// Synchronises the stream and reads the kernels' error word.
gpe_status sync_and_check(gpe_handle h)
{
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    int err = 0;
    GPE_CUDA_TRY(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err != 0) {
        cudaMemsetAsync(h->err, 0, sizeof(int), h->stream);
        cudaStreamSynchronize(h->stream);
        h->epoch_reset = true;  // the persistent kernel's epoch words stopped part-way
        return fail(GPE_ERR_TIMEOUT, "a bounded wait in the fused kernel ran out; the step was abandoned");
    }
    return GPE_OK;
}

// Per-axis trap tables, dt-scaled, rounded to the handle's precision:
// Vx[s][i] = 0.5*trap[0]*x^2 at the value's x position, etc.
void build_trap_tables(const gpe_handle_ &h, int ii, std::vector<double> &out)
{
    const gpe_instance &in = h.inst[ii];
    const int n[3] = {in.nx, in.ny, in.nz};
    out.clear();
    for (int axis = 0; axis < 3; axis++)
        for (int s = 0; s < h.ns; s++)
            for (int i = 0; i < n[axis]; i++) {
                const double p = in.origin[axis] + in.block_scale * (i * h.lat.block_width + h.lat.position[s][axis]);
                out.push_back(0.5 * in.trap[axis] * p * p * in.dt);
            }
}

gpe_status upload_raw(gpe_handle h, const void *src, size_t bytes)
{
    GPE_CUDA_TRY(cudaMemcpyAsync(h->staging, src, bytes, cudaMemcpyHostToDevice, h->stream));
    return GPE_OK;
}

// A host buffer [p, p + bytes) that the conversion kernels can read or write in
// place: page-locked memory mapped into the address space of `device` (cudaHostAlloc,
// cudaHostRegister, made on that device), the whole range inside one such
// allocation, aligned for the kernels' vector accesses.  Returns its device address, or nullptr, in which
// case the transfer goes through device staging and the copy engine.  The
// conversions then move the data over the host link themselves (one pass, no
// staging copy), which on a GPU whose host link is coherent (NVLink-C2C) is
// also the faster path.
using PointerGetAttribute = CUresult (*)(void *, CUpointer_attribute, CUdeviceptr);
static PointerGetAttribute pointer_get_attribute()
{
    static PointerGetAttribute fn = nullptr;
    static bool looked = false;
    if (!looked) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess && f)
            fn = (PointerGetAttribute)f;
        looked = true;
    }
    return fn;
}

void *mapped_host_range(const void *p, size_t bytes, size_t align, int device)
{
    if (!p || bytes == 0) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory on older drivers
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || a.hostPointer != p || a.device != device) return nullptr;
    if (reinterpret_cast<uintptr_t>(a.devicePointer) % align) return nullptr;
    PointerGetAttribute get = pointer_get_attribute();
    if (!get) return nullptr;
    CUdeviceptr start = 0;
    size_t size = 0;
    const CUdeviceptr dp = reinterpret_cast<CUdeviceptr>(a.devicePointer);
    if (get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, dp) != CUDA_SUCCESS ||
        get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, dp) != CUDA_SUCCESS)
        return nullptr;
    if (dp < start || dp - start > size || bytes > size - (dp - start)) return nullptr;
    return a.devicePointer;
}

// Copies the slots in `mask` of one block plane: each slot's values are one
// contiguous run of the padded layout, and neighbouring slots merge.
gpe_status copy_plane_slots(gpe_handle h, char *f, long long dst_plane, long long src_plane, long long slot_len,
                            uint32_t mask)
{
    const size_t cb = 2 * h->esize;
    for (int s = 0; s < h->ns;) {
        if (!(mask >> s & 1u)) {
            s++;
            continue;
        }
        int e = s;
        while (e < h->ns && (mask >> e & 1u)) e++;
        GPE_CUDA_TRY(cudaMemcpyAsync(f + size_t(dst_plane + s * slot_len) * cb, f + size_t(src_plane + s * slot_len) * cb,
                                     size_t(e - s) * size_t(slot_len) * cb, cudaMemcpyDeviceToDevice, h->stream));
        s = e;
    }
    return GPE_OK;
}

// Halo exchange between z-linked instances for one field (the reference's
// z-slab copies, GPUGrossPitaevskii_BCC_multi.cu:660-707 and the slot packing of
// GPUGrossPitaevskii_BCC_MPI.cu:220-271): the lower slab's top interior plane
// feeds the upper slab's bottom padding plane and the upper slab's bottom plane
// the lower slab's top padding plane, each with only the slots the stencil reads
// across that face (TETRA12: 4 and 2 of 12; BCC2: both).
gpe_status enqueue_halo(gpe_handle h, int field)
{
    for (auto &lk : h->zlinks) {
        const InstDev &lo = h->idev_host[lk.first], &up = h->idev_host[lk.second];
        char *f = (char *)field_buf(h, field);
        gpe_status st = copy_plane_slots(h, f, up.base, lo.base + lo.nz * lo.zstride, lo.plane, h->slots_from_below);
        if (st != GPE_OK) return st;
        st = copy_plane_slots(h, f, lo.base + (lo.nz + 1) * lo.zstride, up.base + up.zstride, lo.plane,
                              h->slots_from_above);
        if (st != GPE_OK) return st;
    }
    return GPE_OK;
}

PlainBatchLaunch plain_batch(gpe_handle h, int mode, void *prev, void *next)
{
    PlainBatchLaunch l{};
    l.lattice = step_lattice(h);
    l.precision = h->cfg.precision;
    l.mode = mode;
    l.potential = h->cfg.potential;
    l.inst = h->idev;
    l.blk_inst = h->pb_inst;
    l.blk_begin = h->pb_begin;
    l.zcs = h->pb_zcs;
    l.blocks = h->pb_blocks;
    l.prev = prev;
    l.next = next;
    l.vpot = h->vpot;
    l.vbase = h->vbase;
    l.imag = h->imag;
    return l;
}

gpe_status enqueue_step_real(gpe_handle h)
{
    if (h->two_step) {
        // both half-steps in one launch, from set `parity` into the other set
        FusedLaunch l{};
        l.precision = h->cfg.precision;
        l.mode = GPE_REAL_TIME;
        l.potential = h->cfg.potential;
        l.tile = h->tile;
        l.inst = h->idev;
        l.items = h->items_dev;
        l.num_items = int(h->items.size());
        l.grid = h->grid;
        l.vpot = h->vpot;
        l.maps = h->maps;
        l.zcmax = h->zcmax;
        l.inject_skip_plane = h->inject;
        l.src = h->parity;
        l.out_e = h->buf[2 * (1 - h->parity)];
        l.out_o = h->buf[2 * (1 - h->parity) + 1];
        l.err = h->err;
        l.num_instances = h->cfg.num_instances;
        GPE_CUDA_TRY(launch_twostep(l, h->stream));
        h->launches++;
        h->parity = 1 - h->parity;
        return GPE_OK;
    }
    // the fused kernels' work items: all, or the run a round trip steps
    const int run_first = h->run_count > 0 ? h->run_first : 0;
    const int run_items = h->run_count > 0 ? h->run_count : h->grid;
    // odd <- even, then even <- odd (GPUGrossPitaevskii_BCC.cu:475-481)
    for (int half = 0; half < 2; half++) {
        void *prev = field_buf(h, half == 0 ? 0 : 1);
        void *next = field_buf(h, half == 0 ? 1 : 0);
        if (h->t12) {
            T12Launch l{};
            l.mode = GPE_REAL_TIME;
            l.potential = h->cfg.potential;
            l.variant = h->tile;
            l.grid = run_items;
            l.src = half == 0 ? 0 : 1;
            l.inject_skip_plane = h->inject;
            l.inst = h->idev;
            l.items = h->items_dev + run_first;
            l.maps = h->maps;
            l.vmaps = h->t12_vmaps;
            l.next = next;
            l.vpot = h->cfg.potential == GPE_POTENTIAL_ARRAY ? h->vbase : h->vpot;
            l.err = h->err;
            std::memcpy(l.tab, h->t12_tab, sizeof(l.tab));
            l.face = h->faces ? 1 : 0;
            GPE_CUDA_TRY(launch_t12_step(l, h->stream));
            h->launches++;
        } else if (h->fused) {
            FusedLaunch l{};
            l.precision = h->cfg.precision;
            l.mode = GPE_REAL_TIME;
            l.potential = h->cfg.potential;
            l.tile = h->tile;
            l.inst = h->idev;
            l.items = h->items_dev + run_first;
            l.num_items = run_items;
            l.grid = run_items;
            l.prev = prev;
            l.next = next;
            l.vpot = h->vpot;
            l.maps = h->maps;
            l.zcmax = h->zcmax;
            l.inject_skip_plane = h->inject;
            l.src = half == 0 ? 0 : 1;
            l.comp = h->comp ? 1 : 0;
            l.next_lo = h->lo[half == 0 ? 1 : 0];
            l.lo_maps = h->lo_maps;
            l.err = h->err;
            l.num_instances = h->cfg.num_instances;
            GPE_CUDA_TRY(launch_fused_step(l, h->stream));
            h->launches++;
        } else if (h->pb_blocks > 0) {
            GPE_CUDA_TRY(launch_plain_step_batch(plain_batch(h, GPE_REAL_TIME, prev, next), h->stream));
            h->launches++;
        } else {
            for (int i = 0; i < h->cfg.num_instances; i++) {
                StepLaunch l{};
                l.lattice = step_lattice(h);
                l.precision = h->cfg.precision;
                l.mode = GPE_REAL_TIME;
                l.potential = h->cfg.potential;
                l.inst = h->idev;
                l.inst_index = i;
                l.nx = h->inst[i].nx;
                l.ny = h->inst[i].ny;
                l.nz = h->inst[i].nz;
                l.slots = h->ns;
                l.prev = prev;
                l.next = next;
                l.vpot = h->vpot;
                l.vbase = h->vbase;
                GPE_CUDA_TRY(launch_plain_step(l, h->stream));
                h->launches++;
            }
        }
        gpe_status st = enqueue_halo(h, half == 0 ? 1 : 0);
        if (st != GPE_OK) return st;
    }
    return GPE_OK;
}

gpe_status enqueue_observables(gpe_handle h, const void *field, int i, double *sums_dev)
{
    ObsLaunch o{};
    o.lattice = h->cfg.lattice;
    o.precision = h->cfg.precision;
    o.potential = h->cfg.potential;
    o.inst = h->idev;
    o.inst_index = i;
    o.nx = h->inst[i].nx;
    o.ny = h->inst[i].ny;
    o.nz = h->inst[i].nz;
    o.slots = h->ns;
    o.field = field;
    o.vpot = h->vpot;
    o.partials = h->obs_partials;
    o.max_ctas = h->obs_max_ctas;
    int ctas = 0;
    GPE_CUDA_TRY(launch_observables(o, h->stream, &ctas));
    GPE_CUDA_TRY(launch_reduce_partials(h->obs_partials, ctas, 6, sums_dev, h->stream));
    h->launches += 2;
    return GPE_OK;
}

// One imaginary-time step for every instance; flips the parity.
gpe_status enqueue_step_imag(gpe_handle h, int parity)
{
    void *prev = h->buf[parity], *next = h->buf[1 - parity];
    if (h->t12) {
        T12Launch l{};
        l.mode = GPE_IMAGINARY_TIME;
        l.potential = h->cfg.potential;
        l.variant = h->tile;
        l.grid = h->grid;
        l.src = parity;
        l.inject_skip_plane = h->inject;
        l.imag = h->imag;
        l.partials = h->partials;
        l.counter = h->counter;
        l.inst_item_begin = h->item_begin_dev;
        l.num_instances = h->cfg.num_instances;
        l.tol = h->tol;
        l.inst = h->idev;
        l.items = h->items_dev;
        l.maps = h->maps;
        l.vmaps = h->t12_vmaps;
        l.next = next;
        l.vpot = h->cfg.potential == GPE_POTENTIAL_ARRAY ? h->vbase : h->vpot;
        l.err = h->err;
        std::memcpy(l.tab, h->t12_tab, sizeof(l.tab));
        l.face = h->faces ? 1 : 0;
        GPE_CUDA_TRY(launch_t12_step(l, h->stream));
        h->launches++;
        return GPE_OK;
    }
    if (h->fused) {
        FusedLaunch l{};
        l.precision = h->cfg.precision;
        l.mode = GPE_IMAGINARY_TIME;
        l.potential = h->cfg.potential;
        l.tile = h->tile;
        l.inst = h->idev;
        l.items = h->items_dev;
        l.num_items = int(h->items.size());
        l.grid = h->grid;
        l.prev = prev;
        l.next = next;
        l.vpot = h->vpot;
        l.maps = h->maps;
        l.zcmax = h->zcmax;
        l.inject_skip_plane = h->inject;
        l.src = parity;
        l.err = h->err;
        l.imag = h->imag;
        l.partials = h->partials;
        l.counter = h->counter;
        l.inst_item_begin = h->item_begin_dev;
        l.num_instances = h->cfg.num_instances;
        l.tol = h->tol;
        GPE_CUDA_TRY(launch_fused_step(l, h->stream));
        h->launches++;
        return GPE_OK;
    }
    for (int i = 0; i < h->cfg.num_instances; i++) {
        double *sums = h->obs_sums + 6 * i;
        gpe_status st = enqueue_observables(h, prev, i, sums);
        if (st != GPE_OK) return st;
        GPE_CUDA_TRY(launch_imag_finalize_plain(sums, h->idev, i, h->imag, h->tol, nullptr, h->stream));
        h->launches++;
    }
    if (h->pb_blocks > 0) {
        GPE_CUDA_TRY(launch_plain_step_batch(plain_batch(h, GPE_IMAGINARY_TIME, prev, next), h->stream));
        h->launches++;
        return GPE_OK;
    }
    for (int i = 0; i < h->cfg.num_instances; i++) {
        StepLaunch l{};
        l.lattice = step_lattice(h);
        l.precision = h->cfg.precision;
        l.mode = GPE_IMAGINARY_TIME;
        l.potential = h->cfg.potential;
        l.inst = h->idev;
        l.inst_index = i;
        l.nx = h->inst[i].nx;
        l.ny = h->inst[i].ny;
        l.nz = h->inst[i].nz;
        l.slots = h->ns;
        l.prev = prev;
        l.next = next;
        l.vpot = h->vpot;
        l.vbase = h->vbase;
        l.imag = h->imag;
        GPE_CUDA_TRY(launch_plain_step(l, h->stream));
        h->launches++;
    }
    return GPE_OK;
}

// Imaginary time: compute sigma of the current field and scale it in place so
// that the stored field is normalised and sigma = 1.
gpe_status imag_normalise(gpe_handle h, bool recompute)
{
    for (int i = 0; i < h->cfg.num_instances; i++) {
        if (recompute) {
            double *sums = h->obs_sums + 6 * i;
            gpe_status st = enqueue_observables(h, h->buf[h->parity], i, sums);
            if (st != GPE_OK) return st;
            GPE_CUDA_TRY(launch_imag_init(sums, h->idev, i, h->imag, h->stream));
        }
        GPE_CUDA_TRY(launch_scale_field(h->cfg.precision, h->idev, i, h->inst[i].nx, h->inst[i].ny, h->inst[i].nz,
                                        h->ns, h->buf[h->parity], h->imag, h->stream));
        h->launches += 1;
    }
    GPE_CUDA_TRY(launch_set_sigma_one(h->imag, h->cfg.num_instances, h->stream));
    h->launches++;
    return GPE_OK;
}

gpe_status imag_prepare(gpe_handle h)
{
    if (h->imag_ready) return GPE_OK;
    gpe_status st = imag_normalise(h, true);
    if (st != GPE_OK) return st;
    h->imag_ready = true;
    return GPE_OK;
}

// Enqueues `steps` steps starting from the current parity.
gpe_status enqueue_steps(gpe_handle h, long long steps)
{
    for (long long k = 0; k < steps; k++) {
        gpe_status st;
        if (h->cfg.mode == GPE_REAL_TIME) {
            st = enqueue_step_real(h);
        } else {
            st = enqueue_step_imag(h, h->parity);
            h->parity = 1 - h->parity;
        }
        if (st != GPE_OK) return st;
    }
    return GPE_OK;
}

// Persistent variants: one cooperative launch per call advances every instance
// by `steps` leapfrog steps (no graphs: there is one launch to replay).
gpe_status run_persistent(gpe_handle h, long long steps)
{
    constexpr long long kMaxSteps = 1ll << 24;  // per launch, so the epoch arithmetic stays far from wrapping
    while (steps > 0) {
        const long long n = std::min(steps, kMaxSteps);
        if (h->epoch_reset) {
            GPE_CUDA_TRY(cudaMemsetAsync(h->done, 0, sizeof(unsigned int) * h->items.size(), h->stream));
            h->epoch = 0;
            h->epoch_reset = false;
        }
        GPE_CUDA_TRY(cudaMemsetAsync(h->ticket, 0, sizeof(unsigned long long), h->stream));
        PersistLaunch l{};
        l.precision = h->cfg.precision;
        l.potential = h->cfg.potential;
        l.variant = fused_persistent_index(h->tile);
        l.comp = h->comp ? 1 : 0;
        l.device = h->cfg.device;
        l.inst = h->idev;
        l.items = h->items_dev;
        l.num_items = int(h->items.size());
        l.maps = h->maps;
        l.lo_maps = h->lo_maps;
        l.field[0] = h->buf[0];
        l.field[1] = h->buf[1];
        l.lo[0] = h->lo[0];
        l.lo[1] = h->lo[1];
        l.vpot = h->vpot;
        l.ticket = h->ticket;
        l.nbr_begin = h->nbr_begin_dev;
        l.nbr = h->nbr_dev;
        l.done = h->done;
        l.epoch0 = h->epoch;
        l.half_steps = int(2 * n);
        l.err = h->err;
        l.inject_skip_plane = h->inject;
        int grid = 0;
        GPE_CUDA_TRY(launch_persistent(l, h->stream, &grid));
        h->launches++;
        h->epoch += unsigned(2 * n);
        steps -= n;
    }
    return GPE_OK;
}

gpe_status run_steps(gpe_handle h, long long steps)
{
    if (h->persistent) return run_persistent(h, steps);
    const long long G = h->cfg.graph_steps == 0 ? 100 : h->cfg.graph_steps;
    if (h->cfg.graph_steps < 0 || steps < G) return enqueue_steps(h, steps);
    long long done = 0;
    while (steps - done >= G) {
        GraphKey key{G, h->parity, h->tol, h->run_first, h->run_count};
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            const int parity0 = h->parity;
            const long long launches0 = h->launches;
            GPE_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            gpe_status st = enqueue_steps(h, G);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
            if (st != GPE_OK) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            h->graphs[key] = exec;
            it = h->graphs.find(key);
            // capture only recorded the launches; restore the host-side state
            h->parity = parity0;
            h->launches = launches0;
        }
        GPE_CUDA_TRY(cudaGraphLaunch(it->second, h->stream));
        // account for the launches inside the graph and the parity it leaves
        const long long per_step = (h->cfg.mode == GPE_REAL_TIME)
                                       ? (h->two_step ? 1 : (h->fused ? 2 : 2ll * h->cfg.num_instances))
                                       : (h->fused ? 1 : 4ll * h->cfg.num_instances);
        h->launches += per_step * G;
        if ((h->cfg.mode == GPE_IMAGINARY_TIME || h->two_step) && (G % 2) == 1) h->parity = 1 - h->parity;
        done += G;
    }
    return enqueue_steps(h, steps - done);
}

void free_handle(gpe_handle h)
{
    if (!h) return;
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second);
    cudaFree(h->idev);
    for (void *b : h->buf) cudaFree(b);
    for (void *b : h->lo) cudaFree(b);
    cudaFree(h->vpot);
    cudaFree(h->vbase);
    cudaFree(h->pb_inst);
    cudaFree(h->pb_begin);
    cudaFree(h->pb_zcs);
    cudaFree(h->items_dev);
    cudaFree(h->item_begin_dev);
    cudaFree(h->nbr_begin_dev);
    cudaFree(h->nbr_dev);
    cudaFree(h->done);
    cudaFree(h->ticket);
    cudaFree(h->imag);
    cudaFree(h->partials);
    cudaFree(h->counter);
    cudaFree(h->obs_partials);
    cudaFree(h->obs_sums);
    cudaFree(h->obs_cta_inst);
    cudaFree(h->obs_cta_begin);
    cudaFree(h->obs_batch_partials);
    cudaFree(h->maps);
    cudaFree(h->lo_maps);
    cudaFree(h->err);
    cudaFree(h->staging);
    cudaFree(h->batch_staging);
    for (cudaEvent_t e : h->xfer_events) cudaEventDestroy(e);
    cudaFree(h->xfer_segs);
    cudaFree(h->t12_vmaps);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->down_stream) cudaStreamDestroy(h->down_stream);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

// The fused kernel hard-wires the BCC2 summation order; check it against the
// geometry-derived table.
bool bcc2_order_matches(const gpe_lattice_info &info)
{
    static const int want[2][14][5] = {
        {{-1, -1, -1, 1, 0}, {0, -1, -1, 1, 0}, {-1, 0, -1, 1, 0}, {0, 0, -1, 1, 0},
         {-1, -1, 0, 1, 0}, {0, -1, 0, 1, 0}, {-1, 0, 0, 1, 0}, {0, 0, 0, 1, 0},
         {0, 0, -1, 0, 1}, {0, -1, 0, 0, 1}, {-1, 0, 0, 0, 1}, {1, 0, 0, 0, 1}, {0, 1, 0, 0, 1}, {0, 0, 1, 0, 1}},
        {{0, 0, 0, 0, 0}, {1, 0, 0, 0, 0}, {0, 1, 0, 0, 0}, {1, 1, 0, 0, 0},
         {0, 0, 1, 0, 0}, {1, 0, 1, 0, 0}, {0, 1, 1, 0, 0}, {1, 1, 1, 0, 0},
         {0, 0, -1, 1, 1}, {0, -1, 0, 1, 1}, {-1, 0, 0, 1, 1}, {1, 0, 0, 1, 1}, {0, 1, 0, 1, 1}, {0, 0, 1, 1, 1}}};
    for (int s = 0; s < 2; s++)
        for (int k = 0; k < 14; k++)
            for (int c = 0; c < 5; c++)
                if (info.entry[s][k][c] != want[s][k][c]) return false;
    return true;
}

}  // namespace

extern "C" {

int32_t gpe_abi_version(void) { return GPE_ABI_VERSION; }

const char *gpe_status_string(gpe_status s)
{
    switch (s) {
    case GPE_OK: return "ok";
    case GPE_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GPE_ERR_CUDA: return "CUDA error";
    case GPE_ERR_OUT_OF_MEMORY: return "out of memory";
    case GPE_ERR_NOT_FINITE: return "non-finite values";
    case GPE_ERR_UNSUPPORTED: return "unsupported";
    case GPE_ERR_TOO_LARGE: return "too large";
    case GPE_ERR_INTERNAL: return "internal error";
    case GPE_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

const char *gpe_last_error(void) { return g_last_error.c_str(); }

static gpe_status gpe_lattice_describe_impl(int32_t lattice, gpe_lattice_info *out)
{
    if (!out) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_lattice_describe: null output");
    if (lattice != GPE_LATTICE_TETRA12 && lattice != GPE_LATTICE_BCC2)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_lattice_describe: unknown lattice");
    gpe_status st = build_lattice(gpe_lattice(lattice), out);
    if (st != GPE_OK) return fail(st, "lattice construction failed its self-check");
    return GPE_OK;
}

gpe_status gpe_lattice_describe(int32_t lattice, gpe_lattice_info *out)
{
    GPE_GUARD(gpe_lattice_describe_impl(lattice, out));
}

static gpe_status gpe_create_impl(const gpe_config *cfg, gpe_handle *out)
{
    if (!cfg || !out) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: null argument");
    *out = nullptr;
    if (cfg->lattice != GPE_LATTICE_TETRA12 && cfg->lattice != GPE_LATTICE_BCC2)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: unknown lattice");
    if (cfg->precision != GPE_FP64 && cfg->precision != GPE_FP32 && cfg->precision != GPE_FP32C)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: unknown precision");
    if (cfg->mode != GPE_REAL_TIME && cfg->mode != GPE_IMAGINARY_TIME)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: unknown time mode");
    if (cfg->potential != GPE_POTENTIAL_ARRAY && cfg->potential != GPE_POTENTIAL_TRAP)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: unknown potential kind");
    if (cfg->kernel < GPE_KERNEL_AUTO || cfg->kernel > GPE_KERNEL_FUSED)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: unknown kernel kind");
    if (cfg->num_instances < 1 || !cfg->instances)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: need at least one instance");
    if (cfg->kernel == GPE_KERNEL_FUSED && cfg->lattice == GPE_LATTICE_TETRA12 && cfg->precision != GPE_FP32)
        return fail(GPE_ERR_UNSUPPORTED, "gpe_create: the fused kernel takes the TETRA12 lattice in GPE_FP32 only "
                                         "(the plain kernel runs FP64)");
    if (cfg->faces) {
        if (cfg->lattice != GPE_LATTICE_TETRA12 || cfg->precision == GPE_FP32C)
            return fail(GPE_ERR_UNSUPPORTED, "gpe_create: a face table needs the TETRA12 lattice and GPE_FP64 or "
                                             "GPE_FP32");
        gpe_status fst = check_face_table(*cfg->faces);
        if (fst != GPE_OK) return fst;
    }
    if (cfg->precision == GPE_FP32C &&
        (cfg->lattice != GPE_LATTICE_BCC2 || cfg->kernel == GPE_KERNEL_PLAIN || cfg->mode != GPE_REAL_TIME ||
         (cfg->tile > 0 && cfg->tile < fused_tile_count() && fused_half_steps(cfg->tile) != 1)))
        return fail(GPE_ERR_UNSUPPORTED, "gpe_create: GPE_FP32C needs the BCC2 lattice, the fused kernel, real "
                                         "time and a one-half-step variant");
    for (int i = 0; i < cfg->num_instances; i++) {
        const gpe_instance &in = cfg->instances[i];
        if (in.nx < 1 || in.ny < 1 || in.nz < 1)
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: instance " + std::to_string(i) + " has an empty grid");
        // blockIdx.z of the plain kernel carries nz*slots; x/y tiles are bounded by int range
        if ((long long)in.nz * (cfg->lattice == GPE_LATTICE_TETRA12 ? 12 : 2) > 65535 || in.nx > (1 << 24) ||
            in.ny > (1 << 24))
            return fail(GPE_ERR_TOO_LARGE, "gpe_create: instance " + std::to_string(i) +
                                               " exceeds the grid limits (nz*slots <= 65535)");
        if (!(in.block_scale > 0.0) || !std::isfinite(in.block_scale) || !(in.dt > 0.0) || !std::isfinite(in.dt) ||
            !std::isfinite(in.g))
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_create: instance " + std::to_string(i) +
                                                      " needs finite block_scale > 0, dt > 0 and finite g");
    }
    gpe_handle h = new (std::nothrow) gpe_handle_();
    if (!h) return fail(GPE_ERR_OUT_OF_MEMORY, "gpe_create: host allocation");
    h->cfg = *cfg;
    h->inst.assign(cfg->instances, cfg->instances + cfg->num_instances);
    h->cfg.instances = h->inst.data();
    h->faces = cfg->faces != nullptr;
    h->cfg.faces = nullptr;  // copied into the per-instance data below
    gpe_status st = build_lattice(gpe_lattice(cfg->lattice), &h->lat);
    if (st != GPE_OK) {
        free_handle(h);
        return fail(st, "lattice construction failed its self-check");
    }
    h->ns = h->lat.slots;
    h->esize = cfg->precision == GPE_FP64 ? 8 : 4;
    h->comp = cfg->precision == GPE_FP32C;
    h->hsize = h->comp ? 8 : h->esize;
    // TETRA12: the fused kernel when asked for, and by default in FP32, in either
    // form (the plain kernel runs FP64).
    h->t12 = cfg->lattice == GPE_LATTICE_TETRA12 &&
             (cfg->kernel == GPE_KERNEL_FUSED || (cfg->kernel == GPE_KERNEL_AUTO && cfg->precision == GPE_FP32));
    h->fused = (cfg->lattice == GPE_LATTICE_BCC2 && cfg->kernel != GPE_KERNEL_PLAIN) || h->t12;
    if (h->t12)
        for (int s = 0; s < 12; s++)
            for (int k = 0; k < 4; k++) {
                const int *e = h->lat.entry[s][k];
                h->t12_tab[s * 4 + k] = (e[0] + 1) | ((e[1] + 1) << 2) | ((e[2] + 1) << 4) | (e[3] << 6);
            }
    if (h->fused && !h->t12 && !bcc2_order_matches(h->lat)) {
        free_handle(h);
        return fail(GPE_ERR_INTERNAL, "BCC2 table order differs from the fused kernel's");
    }
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "cudaSetDevice");
    }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        gpe_status s2 = cuda_fail(e, "cudaStreamCreate");
        free_handle(h);
        return s2;
    }
#define GPE_CREATE_TRY(expr)                           \
    do {                                               \
        cudaError_t e_ = (expr);                       \
        if (e_ != cudaSuccess) {                       \
            gpe_status s_ = cuda_fail(e_, #expr);      \
            free_handle(h);                            \
            return s_;                                 \
        }                                              \
    } while (0)
    GPE_CREATE_TRY(set_plain_table(h->lat));

    // Arena layout.
    size_t off = 0, voff = 0, max_vals = 0, out_bytes = 0;
    std::vector<std::vector<double>> traps(cfg->num_instances);
    for (int i = 0; i < cfg->num_instances; i++) {
        const gpe_instance &in = h->inst[i];
        InstDev d{};
        d.nx = in.nx;
        d.ny = in.ny;
        d.nz = in.nz;
        // rows start on 16 bytes: 4 values (8 for GPE_FP32C, whose 16-bit
        // residual rows have the same pitch).  A pitch of 16 values for
        // GPE_FP32C, which puts every residual row on a 32-byte sector, measured
        // 9% more DRAM reads per half-step on the 64-condensate batch.
        d.px = int(round_up(size_t(in.nx) + kPadX + 1, h->comp ? 8 : 4));
        d.py = in.ny + 2;
        d.slots = h->ns;
        d.plane = (long long)d.px * d.py;
        d.zstride = (long long)h->ns * d.plane;
        d.base = (long long)off;
        off += round_up(size_t(d.zstride) * (in.nz + 2), 64);
        if (cfg->potential == GPE_POTENTIAL_ARRAY) {
            d.vbase = (long long)voff;
            voff += round_up(size_t(d.zstride) * (in.nz + 2), 64);
        } else {
            build_trap_tables(*h, i, traps[i]);
            d.vbase = (long long)voff;
            voff += round_up(traps[i].size(), 64);
        }
        const double s2 = in.block_scale * in.block_scale;
        d.w[0] = h->lat.class_weight[0] / s2;
        d.w[1] = h->lat.classes > 1 ? h->lat.class_weight[1] / s2 : 0.0;
        d.Lc[0] = -0.5 * d.w[0] * in.dt;
        d.Lc[1] = -0.5 * d.w[1] * in.dt;
        // L0 = (0.5 * sum_c n_c w_c) * dt, classes in order; for TETRA12 this is
        // the reference's lapfac0 = 4 * 0.5 * hodge / bs^2, times dt (:291-306).
        int ncls[2] = {0, 0};
        for (int k = 0; k < h->lat.neighbours; k++) ncls[h->lat.entry[0][k][4]]++;
        double wsum = ncls[0] * d.w[0];
        if (h->lat.classes > 1) wsum = wsum + ncls[1] * d.w[1];
        d.L0 = (0.5 * wsum) * in.dt;
        d.gdt = in.g * in.dt;
        d.dt = in.dt;
        d.g = in.g;
        d.vol = h->lat.cell_volume * in.block_scale * in.block_scale * in.block_scale;
        if (cfg->faces) {
            const gpe_face_table &t = *cfg->faces;
            d.face = 1;
            for (int sl = 0; sl < 12; sl++)
                for (int k = 0; k < 4; k++) {
                    const int f = 4 * sl + kFacePerm[sl][k], j = 4 * sl + k;
                    d.fe[j] = (t.dir[f][0] + 1) | ((t.dir[f][1] + 1) << 2) | ((t.dir[f][2] + 1) << 4) | (t.slot[f] << 6);
                    d.hf[j] = -0.5 * t.hodge[f] / s2 * in.dt;  // GPUGrossPitaevskii_BCC_multi.cu:483
                    d.hf32[j] = float(d.hf[j]);
                    d.hw[j] = t.hodge[f] / s2;
                }
        }
        h->idev_host.push_back(d);
        max_vals = std::max(max_vals, size_t(in.nx) * in.ny * in.nz * h->ns);
        // the output kernels stage a padded block grid of uint16 / a padded plane of RGB
        out_bytes = std::max(out_bytes, size_t(in.nx + 2) * (in.ny + 2) * (in.nz + 2) * 2);
        out_bytes = std::max(out_bytes, size_t(in.nx + 2) * (in.ny + 2) * 3);
    }
    h->field_elems = off;
    h->v_elems = voff;
    const size_t cbytes = 2 * h->esize;
    // Every set-up copy and fill below is ordered on the handle's own
    // (non-blocking) stream: a non-blocking stream does not synchronise with the
    // legacy default stream, so mixing cudaMemcpy with cudaMemsetAsync here would
    // let a fill overwrite a copy.  Host sources stay alive until the final
    // stream synchronisation.
    GPE_CREATE_TRY(cudaMalloc(&h->idev, sizeof(InstDev) * h->idev_host.size()));
    GPE_CREATE_TRY(cudaMemcpyAsync(h->idev, h->idev_host.data(), sizeof(InstDev) * h->idev_host.size(),
                                   cudaMemcpyHostToDevice, h->stream));
    GPE_CREATE_TRY(cudaMalloc(&h->buf[0], cbytes * h->field_elems));
    GPE_CREATE_TRY(cudaMalloc(&h->buf[1], cbytes * h->field_elems));
    GPE_CREATE_TRY(cudaMemsetAsync(h->buf[0], 0, cbytes * h->field_elems, h->stream));
    GPE_CREATE_TRY(cudaMemsetAsync(h->buf[1], 0, cbytes * h->field_elems, h->stream));
    if (h->comp)
        for (int f = 0; f < 2; f++) {
            GPE_CREATE_TRY(cudaMalloc(&h->lo[f], sizeof(uint16_t) * h->field_elems));
            GPE_CREATE_TRY(cudaMemsetAsync(h->lo[f], 0, sizeof(uint16_t) * h->field_elems, h->stream));
        }
    GPE_CREATE_TRY(cudaMalloc(&h->vpot, h->esize * std::max<size_t>(h->v_elems, 1)));
    GPE_CREATE_TRY(cudaMemsetAsync(h->vpot, 0, h->esize * std::max<size_t>(h->v_elems, 1), h->stream));
    if (cfg->potential == GPE_POTENTIAL_ARRAY) {
        GPE_CREATE_TRY(cudaMalloc(&h->vbase, h->esize * std::max<size_t>(h->v_elems, 1)));
        GPE_CREATE_TRY(cudaMemsetAsync(h->vbase, 0, h->esize * std::max<size_t>(h->v_elems, 1), h->stream));
    }
    std::vector<std::vector<float>> traps32(cfg->num_instances);
    if (cfg->potential == GPE_POTENTIAL_TRAP) {
        for (int i = 0; i < cfg->num_instances; i++) {
            const size_t n = traps[i].size();
            if (cfg->precision == GPE_FP64) {
                GPE_CREATE_TRY(cudaMemcpyAsync((double *)h->vpot + h->idev_host[i].vbase, traps[i].data(), 8 * n,
                                               cudaMemcpyHostToDevice, h->stream));
            } else {
                traps32[i].assign(traps[i].begin(), traps[i].end());
                GPE_CREATE_TRY(cudaMemcpyAsync((float *)h->vpot + h->idev_host[i].vbase, traps32[i].data(), 4 * n,
                                               cudaMemcpyHostToDevice, h->stream));
            }
        }
    }
    h->staging_bytes = std::max<size_t>(std::max(max_vals * 2 * h->hsize, out_bytes), 64);
    GPE_CREATE_TRY(cudaMalloc(&h->staging, h->staging_bytes));
    GPE_CREATE_TRY(cudaMalloc(&h->imag, sizeof(ImagScalars) * cfg->num_instances));
    std::vector<ImagScalars> imag_init(cfg->num_instances);
    for (auto &sc : imag_init) {
        sc = ImagScalars{};
        sc.sigma = 1.0;
        sc.conv_step = -1;
    }
    GPE_CREATE_TRY(cudaMemcpyAsync(h->imag, imag_init.data(), sizeof(ImagScalars) * imag_init.size(),
                                   cudaMemcpyHostToDevice, h->stream));
    GPE_CREATE_TRY(cudaMalloc(&h->err, sizeof(int)));
    GPE_CREATE_TRY(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
    GPE_CREATE_TRY(cudaMalloc(&h->obs_partials, sizeof(double) * 6 * h->obs_max_ctas));
    GPE_CREATE_TRY(cudaMalloc(&h->obs_sums, sizeof(double) * 6 * cfg->num_instances));
    std::vector<int> cta_begin(cfg->num_instances + 1, 0), cta_inst;
    for (int i = 0; i < cfg->num_instances; i++) {
        const gpe_instance &in = h->inst[i];
        const int c = observables_batch_ctas((long long)in.nx * in.ny * in.nz * h->ns, h->obs_max_ctas);
        cta_begin[i + 1] = cta_begin[i] + c;
        cta_inst.insert(cta_inst.end(), size_t(c), i);
    }
    h->obs_total_ctas = cta_begin.back();
    GPE_CREATE_TRY(cudaMalloc(&h->obs_cta_inst, sizeof(int) * cta_inst.size()));
    GPE_CREATE_TRY(cudaMalloc(&h->obs_cta_begin, sizeof(int) * cta_begin.size()));
    GPE_CREATE_TRY(cudaMalloc(&h->obs_batch_partials, sizeof(double) * 6 * size_t(h->obs_total_ctas)));
    GPE_CREATE_TRY(cudaMemcpyAsync(h->obs_cta_inst, cta_inst.data(), sizeof(int) * cta_inst.size(),
                                   cudaMemcpyHostToDevice, h->stream));
    GPE_CREATE_TRY(cudaMemcpyAsync(h->obs_cta_begin, cta_begin.data(), sizeof(int) * cta_begin.size(),
                                   cudaMemcpyHostToDevice, h->stream));
    // The plain kernel over a batch: one launch per half-step for all instances.
    std::vector<int> pb_begin, pb_inst, pb_zcs;
    if (!h->fused && cfg->num_instances > 1) {
        pb_begin.assign(cfg->num_instances + 1, 0);
        for (int i = 0; i < cfg->num_instances; i++) {
            const gpe_instance &in = h->inst[i];
            const int zc = plain_planes_per_thread((long long)in.nx * in.ny * in.nz * h->ns, cfg->precision);
            const long long blocks = (long long)plain_blocks_per_plane(in.nx, in.ny) * ((in.nz + zc - 1) / zc) * h->ns;
            if ((long long)pb_begin[i] + blocks > 0x7fffffffll) {
                pb_begin.clear();
                break;  // too many CTAs for one launch: keep one launch per instance
            }
            pb_begin[i + 1] = pb_begin[i] + int(blocks);
            pb_inst.insert(pb_inst.end(), size_t(blocks), i);
            pb_zcs.push_back(zc);
        }
        if (!pb_begin.empty()) {
            h->pb_blocks = pb_begin.back();
            GPE_CREATE_TRY(cudaMalloc(&h->pb_inst, sizeof(int) * pb_inst.size()));
            GPE_CREATE_TRY(cudaMalloc(&h->pb_begin, sizeof(int) * pb_begin.size()));
            GPE_CREATE_TRY(cudaMalloc(&h->pb_zcs, sizeof(int) * pb_zcs.size()));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->pb_inst, pb_inst.data(), sizeof(int) * pb_inst.size(),
                                           cudaMemcpyHostToDevice, h->stream));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->pb_begin, pb_begin.data(), sizeof(int) * pb_begin.size(),
                                           cudaMemcpyHostToDevice, h->stream));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->pb_zcs, pb_zcs.data(), sizeof(int) * pb_zcs.size(),
                                           cudaMemcpyHostToDevice, h->stream));
        }
    }
    GPE_CREATE_TRY(cudaStreamSynchronize(h->stream));  // the host tables above go out of scope

    if (h->t12) {
        int st_;
        h->tile = cfg->tile > 0 && cfg->tile < t12_variant_count() ? cfg->tile : 0;
        t12_variant(h->tile, &h->tx, &h->ty, &st_);
    } else if (h->fused) {
        h->tile = cfg->tile > 0 && cfg->tile < fused_tile_count() ? cfg->tile : 0;
        fused_tile_shape(h->tile, &h->tx, &h->ty);
    }
    if (h->fused) {
        if (!h->t12 && fused_variant_kind(h->tile) == kVariantPersistent) {
            if (cfg->mode != GPE_REAL_TIME) {
                free_handle(h);
                return fail(GPE_ERR_UNSUPPORTED, "gpe_create: the persistent kernel variants advance real time; "
                                                 "imaginary time needs a one-launch-per-half-step variant");
            }
            h->persistent = true;
        }
        if (!h->t12 && fused_half_steps(h->tile) == 2) {
            if (cfg->mode != GPE_REAL_TIME) {
                free_handle(h);
                return fail(GPE_ERR_UNSUPPORTED, "gpe_create: this kernel variant advances whole real-time steps; "
                                                 "imaginary time needs a half-step variant");
            }
            h->two_step = true;
            for (int b = 2; b < 4; b++) {
                GPE_CREATE_TRY(cudaMalloc(&h->buf[b], cbytes * h->field_elems));
                GPE_CREATE_TRY(cudaMemsetAsync(h->buf[b], 0, cbytes * h->field_elems, h->stream));
            }
        }
        // Instances in decreasing size; each instance's items contiguous,
        // x fastest, then y, then z-chunk.
        std::vector<int> order(cfg->num_instances);
        for (int i = 0; i < cfg->num_instances; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const gpe_instance &A = h->inst[a], &B = h->inst[b];
            return (long long)A.nx * A.ny * A.nz > (long long)B.nx * B.ny * B.nz;
        });
        int zc = cfg->zchunk;
        if (zc <= 0) {
            // Real time: aim for >= ~4 waves of 152 SMs x 8 CTAs, halving the chunk
            // down to 2 planes: a small grid needs short chunks to occupy the GPU
            // (one 32^3 instance: 1.45e10 vertex-updates/s with 2-plane chunks,
            // 1.01e10 with 8).  Imaginary time pays a reduction per item and a final
            // fold over all items every step, so it aims for about two items per SM
            // and keeps chunks of at least 8 planes.
            const bool imag = cfg->mode == GPE_IMAGINARY_TIME;
            // (the TETRA12 kernel runs one CTA per SM: four waves of 152)
            const long long target = imag ? 152ll * 2 : (h->t12 ? 152ll * 4 : 152ll * 8 * 4);
            const int zmin = imag ? 8 : 2;
            long long maxnz = 1;
            for (auto &in : h->inst) maxnz = std::max<long long>(maxnz, in.nz);
            zc = int(maxnz);
            while (zc > zmin) {
                long long items = 0;
                for (auto &in : h->inst)
                    items += (long long)((in.nx + h->tx - 1) / h->tx) * ((in.ny + h->ty - 1) / h->ty) *
                             ((in.nz + zc - 1) / zc);
                if (items >= target) break;
                zc = (zc + 1) / 2;
            }
            if (zc < zmin) zc = int(std::min<long long>(zmin, maxnz));
            if (!imag && zc < 8 && maxnz >= 8) {
                // below 8 planes the two halo planes of every item weigh more: go
                // back to 8 wherever 8 still gives about four items per SM
                long long items8 = 0;
                for (auto &in : h->inst)
                    items8 += (long long)((in.nx + h->tx - 1) / h->tx) * ((in.ny + h->ty - 1) / h->ty) *
                              ((in.nz + 7) / 8);
                if (items8 >= 152ll * 4) zc = 8;
            }
        }
        h->zchunk = zc;
        h->zcmax = 1;
        for (auto &in : h->inst) h->zcmax = std::max(h->zcmax, std::min(in.nz, zc));
        std::vector<std::vector<WorkItem>> per(cfg->num_instances);
        for (int i = 0; i < cfg->num_instances; i++) {
            const gpe_instance &in = h->inst[i];
            for (int z0 = 0; z0 < in.nz; z0 += zc)
                for (int y0 = 0; y0 < in.ny; y0 += h->ty)
                    for (int x0 = 0; x0 < in.nx; x0 += h->tx)
                        per[i].push_back(WorkItem{i, x0, y0, z0, std::min(in.nz, z0 + zc)});
        }
        std::vector<int> first(cfg->num_instances);
        for (int oi : order) {
            first[oi] = int(h->items.size());
            h->items.insert(h->items.end(), per[oi].begin(), per[oi].end());
        }
        h->item_order = order;
        h->item_first = first;
        h->item_count.resize(cfg->num_instances);
        for (int i = 0; i < cfg->num_instances; i++) h->item_count[i] = int(per[i].size());
        if (h->persistent) {
            // Each item depends on the items of its instance within one tile and
            // one z-chunk (itself included): the halo it reads, and the reads of
            // the field it rewrites.  Items of instance i are numbered
            // first[i] + (zi * nty + yi) * ntx + xi.
            std::vector<int> nb_begin(1, 0), nb;
            std::vector<int> owner(h->items.size());
            for (int i = 0; i < cfg->num_instances; i++)
                for (size_t k = 0; k < per[i].size(); k++) owner[first[i] + k] = i;
            for (size_t it = 0; it < h->items.size(); it++) {
                const int i = owner[it];
                const gpe_instance &in = h->inst[i];
                const int ntx = (in.nx + h->tx - 1) / h->tx, nty = (in.ny + h->ty - 1) / h->ty;
                const int nzc = (in.nz + zc - 1) / zc;
                const WorkItem &w = h->items[it];
                const int xi = w.x0 / h->tx, yi = w.y0 / h->ty, zi = w.z0 / zc;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            const int X = xi + dx, Y = yi + dy, Z = zi + dz;
                            if (X < 0 || X >= ntx || Y < 0 || Y >= nty || Z < 0 || Z >= nzc) continue;
                            nb.push_back(first[i] + (Z * nty + Y) * ntx + X);
                        }
                nb_begin.push_back(int(nb.size()));
            }
            GPE_CREATE_TRY(cudaMalloc(&h->nbr_begin_dev, sizeof(int) * nb_begin.size()));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->nbr_begin_dev, nb_begin.data(), sizeof(int) * nb_begin.size(),
                                           cudaMemcpyHostToDevice, h->stream));
            GPE_CREATE_TRY(cudaMalloc(&h->nbr_dev, sizeof(int) * nb.size()));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->nbr_dev, nb.data(), sizeof(int) * nb.size(), cudaMemcpyHostToDevice,
                                           h->stream));
            GPE_CREATE_TRY(cudaMalloc(&h->ticket, sizeof(unsigned long long)));
            GPE_CREATE_TRY(cudaMalloc(&h->done, sizeof(unsigned int) * h->items.size()));
            GPE_CREATE_TRY(cudaMemsetAsync(h->done, 0, sizeof(unsigned int) * h->items.size(), h->stream));
        }
        // Items of instance i occupy rows [first[i], first[i] + per[i].size()).
        std::vector<int> ranges(2 * cfg->num_instances);
        for (int i = 0; i < cfg->num_instances; i++) {
            ranges[2 * i] = first[i];
            ranges[2 * i + 1] = first[i] + int(per[i].size());
        }
        // TMA maps: per instance and field (halo box, interior box); for the
        // two-step variants per instance and buffer set (E box, O box).
        std::vector<CUtensorMap> maps(4 * cfg->num_instances);
        for (int i = 0; i < cfg->num_instances; i++)
            for (int f = 0; f < 2; f++) {
                gpe_status ms = h->t12 ? make_t12_maps(&maps[4 * i + 2 * f], h->idev_host[i], h->buf[f], h->tx, h->ty)
                                : h->two_step ? make_twostep_maps(&maps[4 * i + 2 * f], cfg->precision, h->idev_host[i],
                                                                  h->buf[2 * f], h->buf[2 * f + 1], h->tile)
                                              : make_halo_map(&maps[4 * i + 2 * f], cfg->precision, h->idev_host[i],
                                                              h->buf[f], h->tile);
                if (ms != GPE_OK) {
                    free_handle(h);
                    return ms;
                }
            }
        GPE_CREATE_TRY(cudaMalloc(&h->maps, sizeof(CUtensorMap) * maps.size()));
        GPE_CREATE_TRY(cudaMemcpyAsync(h->maps, maps.data(), sizeof(CUtensorMap) * maps.size(),
                                       cudaMemcpyHostToDevice, h->stream));
        if (h->t12 && cfg->potential == GPE_POTENTIAL_ARRAY) {
            std::vector<CUtensorMap> vmaps(cfg->num_instances);
            for (int i = 0; i < cfg->num_instances; i++) {
                // the face form adds V dt itself; the lattice form reads L0 + V dt
                gpe_status ms = make_t12_vmap(&vmaps[i], h->idev_host[i], h->faces ? h->vpot : h->vbase, h->tx,
                                              h->ty);
                if (ms != GPE_OK) {
                    free_handle(h);
                    return ms;
                }
            }
            GPE_CREATE_TRY(cudaMalloc(&h->t12_vmaps, sizeof(CUtensorMap) * vmaps.size()));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->t12_vmaps, vmaps.data(), sizeof(CUtensorMap) * vmaps.size(),
                                           cudaMemcpyHostToDevice, h->stream));
        }
        std::vector<CUtensorMap> lo_maps(h->comp ? 2 * cfg->num_instances : 0);
        for (int i = 0; i < int(lo_maps.size()) / 2; i++)
            for (int f = 0; f < 2; f++) {
                gpe_status ms = make_residual_map(&lo_maps[2 * i + f], h->idev_host[i], h->lo[f], h->tile);
                if (ms != GPE_OK) {
                    free_handle(h);
                    return ms;
                }
            }
        if (!lo_maps.empty()) {
            GPE_CREATE_TRY(cudaMalloc(&h->lo_maps, sizeof(CUtensorMap) * lo_maps.size()));
            GPE_CREATE_TRY(cudaMemcpyAsync(h->lo_maps, lo_maps.data(), sizeof(CUtensorMap) * lo_maps.size(),
                                           cudaMemcpyHostToDevice, h->stream));
        }
        GPE_CREATE_TRY(cudaMalloc(&h->items_dev, sizeof(WorkItem) * h->items.size()));
        GPE_CREATE_TRY(cudaMemcpyAsync(h->items_dev, h->items.data(), sizeof(WorkItem) * h->items.size(),
                                       cudaMemcpyHostToDevice, h->stream));
        GPE_CREATE_TRY(cudaMalloc(&h->item_begin_dev, sizeof(int) * ranges.size()));
        GPE_CREATE_TRY(cudaMemcpyAsync(h->item_begin_dev, ranges.data(), sizeof(int) * ranges.size(),
                                       cudaMemcpyHostToDevice, h->stream));
        h->grid = int(h->items.size());
        if (cfg->mode == GPE_IMAGINARY_TIME) {
            GPE_CREATE_TRY(cudaMalloc(&h->partials, sizeof(double) * 4 * h->items.size()));
            GPE_CREATE_TRY(cudaMalloc(&h->counter, sizeof(unsigned int)));
            GPE_CREATE_TRY(cudaMemsetAsync(h->counter, 0, sizeof(unsigned int), h->stream));
        }
        // ranges must outlive the copy above
        e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) {
            gpe_status s2 = cuda_fail(e, "gpe_create: initialisation");
            free_handle(h);
            return s2;
        }
    }
#undef GPE_CREATE_TRY
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        gpe_status s2 = cuda_fail(e, "gpe_create: initialisation");
        free_handle(h);
        return s2;
    }
    *out = h;
    return GPE_OK;
}

gpe_status gpe_create(const gpe_config *cfg, gpe_handle *out)
{
    GPE_GUARD(gpe_create_impl(cfg, out));
}

static gpe_status gpe_destroy_impl(gpe_handle h)
{
    if (!h) return GPE_OK;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    free_handle(h);
    if (e != cudaSuccess) return cuda_fail(e, "gpe_destroy");
    return GPE_OK;
}

gpe_status gpe_destroy(gpe_handle h)
{
    GPE_GUARD(gpe_destroy_impl(h));
}

static gpe_status gpe_upload_impl(gpe_handle h, int32_t instance, const void *even, const void *odd, const void *potential)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (instance < 0 || instance >= h->cfg.num_instances) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload: bad instance");
    if (!even) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload: even field is required");
    if (h->cfg.mode == GPE_REAL_TIME && !odd)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload: odd field is required in real time");
    if (h->cfg.potential == GPE_POTENTIAL_ARRAY && !potential)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload: potential array is required");
    const gpe_instance &in = h->inst[instance];
    const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
    const int prec = h->cfg.precision;
    const void *srcs[2] = {even, odd};
    for (int f = 0; f < 2; f++) {
        if (!srcs[f]) continue;
        const size_t b = vals * 2 * h->hsize;
        const void *src = mapped_host_range(srcs[f], b, 2 * h->hsize, h->cfg.device);
        if (src) h->mapped_transfers++;
        if (!src) {
            st = upload_raw(h, srcs[f], b);
            if (st != GPE_OK) return st;
            src = h->staging;
        }
        if (h->comp)
            GPE_CUDA_TRY(launch_pack_split(h->idev, instance, in.nx, in.ny, in.nz, h->ns, src, field_buf(h, f),
                                           h->lo[f], h->host_fp32, h->stream));
        else
            GPE_CUDA_TRY(launch_pack(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, src, field_buf(h, f), 1, 1.0,
                                     h->stream));
        h->launches++;
        GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    if (h->cfg.potential == GPE_POTENTIAL_ARRAY) {
        const void *src = mapped_host_range(potential, vals * h->esize, h->esize, h->cfg.device);
        if (src) h->mapped_transfers++;
        if (!src) {
            st = upload_raw(h, potential, vals * h->esize);
            if (st != GPE_OK) return st;
            src = h->staging;
        }
        GPE_CUDA_TRY(launch_pack(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, src, h->vpot, 0, in.dt,
                                 h->stream));
        GPE_CUDA_TRY(launch_potential_base(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, h->vpot, h->vbase,
                                           h->stream));
        h->launches += 2;
    }
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->imag_ready = false;
    return GPE_OK;
}

gpe_status gpe_upload(gpe_handle h, int32_t instance, const void *even, const void *odd, const void *potential)
{
    GPE_GUARD(gpe_upload_impl(h, instance, even, odd, potential));
}

static gpe_status gpe_download_impl(gpe_handle h, int32_t instance, void *even, void *odd)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (instance < 0 || instance >= h->cfg.num_instances)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_download: bad instance");
    st = sync_and_check(h);
    if (st != GPE_OK) return st;
    const gpe_instance &in = h->inst[instance];
    const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
    void *dsts[2] = {even, odd};
    for (int f = 0; f < 2; f++) {
        if (!dsts[f]) continue;
        const size_t b = vals * 2 * h->hsize;
        void *mapped = mapped_host_range(dsts[f], b, 2 * h->hsize, h->cfg.device);
        if (mapped) h->mapped_transfers++;
        void *out = mapped ? mapped : h->staging;
        if (h->comp)
            GPE_CUDA_TRY(launch_unpack_join(h->idev, instance, in.nx, in.ny, in.nz, h->ns, field_buf(h, f), h->lo[f],
                                            out, h->host_fp32, h->stream));
        else
            GPE_CUDA_TRY(launch_unpack(h->cfg.precision, h->idev, instance, in.nx, in.ny, in.nz, h->ns,
                                       field_buf(h, f), out, nullptr, h->stream));
        h->launches++;
        if (!mapped) GPE_CUDA_TRY(cudaMemcpyAsync(dsts[f], h->staging, b, cudaMemcpyDeviceToHost, h->stream));
        GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    return GPE_OK;
}

gpe_status gpe_download(gpe_handle h, int32_t instance, void *even, void *odd)
{
    GPE_GUARD(gpe_download_impl(h, instance, even, odd));
}

namespace {

// Device buffer of at least `bytes` for the batched transfers, grown on demand.
gpe_status ensure_batch_staging(gpe_handle h, size_t bytes)
{
    if (h->batch_bytes >= bytes) return GPE_OK;
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    cudaFree(h->batch_staging);
    h->batch_staging = nullptr;
    h->batch_bytes = 0;
    GPE_CUDA_TRY(cudaMalloc(&h->batch_staging, bytes));
    h->batch_bytes = bytes;
    return GPE_OK;
}

size_t slot_bytes(size_t b) { return round_up(b, 256); }

// The copy stream and at least n events for one batched transfer.
gpe_status ensure_xfer(gpe_handle h, size_t n)
{
    if (!h->copy_stream) GPE_CUDA_TRY(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    while (h->xfer_events.size() < n) {
        cudaEvent_t e;
        GPE_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        h->xfer_events.push_back(e);
    }
    return GPE_OK;
}

// One launch converting every listed (instance, field) between its mapped host
// buffer and the device layout, on the handle's stream (segments in order).
gpe_status run_xfer_batch(gpe_handle h, bool up, const std::vector<std::tuple<const void *, int, int>> &items)
{
    std::vector<XferSeg> &segs = h->xfer_segs_host;
    segs.clear();
    int cta = 0;
    for (const auto &it : items) {
        const gpe_instance &in = h->inst[std::get<1>(it)];
        const long long vals = (long long)in.nx * in.ny * in.nz * h->ns;
        segs.push_back({std::get<0>(it), std::get<1>(it), std::get<2>(it), cta, 0});
        cta += int((vals + kXferValuesPerCta - 1) / kXferValuesPerCta);
    }
    segs.push_back({nullptr, 0, 0, cta, 0});
    if (segs.size() > h->xfer_segs_cap) {
        cudaFree(h->xfer_segs);
        h->xfer_segs = nullptr;
        h->xfer_segs_cap = 0;
        GPE_CUDA_TRY(cudaMalloc(&h->xfer_segs, sizeof(XferSeg) * segs.size()));
        h->xfer_segs_cap = segs.size();
    }
    GPE_CUDA_TRY(cudaMemcpyAsync(h->xfer_segs, segs.data(), sizeof(XferSeg) * segs.size(), cudaMemcpyHostToDevice,
                                 h->stream));
    GPE_CUDA_TRY(launch_xfer_batch(h->cfg.precision, h->comp, h->host_fp32, up, h->idev, h->xfer_segs,
                                   int(segs.size()) - 1, cta, field_buf(h, 0), field_buf(h, 1), h->lo[0], h->lo[1],
                                   h->stream));
    h->launches++;
    h->mapped_transfers += (long long)items.size();
    return GPE_OK;
}

}  // namespace

static gpe_status gpe_upload_many_impl(gpe_handle h, int32_t count, const int32_t *instances, const void *const *even,
                                       const void *const *odd, const void *const *potential)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (count < 0 || (count > 0 && (!instances || !even)))
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload_many: bad count or null array");
    const bool arr = h->cfg.potential == GPE_POTENTIAL_ARRAY;
    // Each buffer in mapped page-locked memory is converted in place (no staging
    // copy); the others are staged.
    std::vector<const void *> mapped(size_t(count) * 3, nullptr);
    size_t total = 0;
    for (int k = 0; k < count; k++) {
        const int i = instances[k];
        if (i < 0 || i >= h->cfg.num_instances) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload_many: bad instance");
        if (!even[k]) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload_many: even field is required");
        if (h->cfg.mode == GPE_REAL_TIME && (!odd || !odd[k]))
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload_many: odd field is required in real time");
        if (arr && (!potential || !potential[k]))
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_upload_many: potential array is required");
        const gpe_instance &in = h->inst[i];
        const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
        const void *bufs[3] = {even[k], odd ? odd[k] : nullptr, arr ? potential[k] : nullptr};
        const size_t bytes[3] = {vals * 2 * h->hsize, vals * 2 * h->hsize, vals * h->esize};
        const size_t align[3] = {2 * h->hsize, 2 * h->hsize, h->esize};
        for (int f = 0; f < 3; f++) {
            if (!bufs[f]) continue;
            mapped[3 * k + f] = mapped_host_range(bufs[f], bytes[f], align[f], h->cfg.device);
            if (!mapped[3 * k + f]) total += slot_bytes(bytes[f]);
        }
    }
    if (total == 0 && !arr) {  // every field in mapped memory: one in-place launch
        std::vector<std::tuple<const void *, int, int>> items;
        for (int k = 0; k < count; k++)
            for (int f = 0; f < 2; f++)
                if (mapped[3 * k + f]) items.emplace_back(mapped[3 * k + f], instances[k], f);
        if (!items.empty() && (st = run_xfer_batch(h, true, items)) != GPE_OK) return st;
        GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
        h->imag_ready = false;
        return GPE_OK;
    }
    st = ensure_batch_staging(h, std::max<size_t>(total, 256));
    if (st == GPE_OK) st = ensure_xfer(h, size_t(3) * count + 1);
    if (st != GPE_OK) return st;
    char *stage = (char *)h->batch_staging;
    const int prec = h->cfg.precision;
    // Copies go on the copy stream back to back; each conversion waits for its
    // own copy on the handle's stream, so conversions overlap later copies.
    // The copy stream first waits for the handle's stream (earlier work).  (The
    // copies spread over four streams measured slower end to end: 10.9 against
    // 9.6 ms of transfers per call on the 64-condensate batch.)
    size_t ev = 0;
    GPE_CUDA_TRY(cudaEventRecord(h->xfer_events[ev], h->stream));
    GPE_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->xfer_events[ev++], 0));
    auto copy_in = [&](void *dst, const void *src, size_t b) -> gpe_status {
        GPE_CUDA_TRY(cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, h->copy_stream));
        GPE_CUDA_TRY(cudaEventRecord(h->xfer_events[ev], h->copy_stream));
        GPE_CUDA_TRY(cudaStreamWaitEvent(h->stream, h->xfer_events[ev++], 0));
        return GPE_OK;
    };
    for (int k = 0; k < count; k++) {
        const int i = instances[k];
        const gpe_instance &in = h->inst[i];
        const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
        const void *srcs[2] = {even[k], odd ? odd[k] : nullptr};
        for (int f = 0; f < 2; f++) {
            if (!srcs[f]) continue;
            const size_t b = vals * 2 * h->hsize;
            const void *src = mapped[3 * k + f];
            if (src) h->mapped_transfers++;
            else {
                if ((st = copy_in(stage, srcs[f], b)) != GPE_OK) return st;
                src = stage;
                stage += slot_bytes(b);
            }
            if (h->comp)
                GPE_CUDA_TRY(launch_pack_split(h->idev, i, in.nx, in.ny, in.nz, h->ns, src, field_buf(h, f), h->lo[f],
                                               h->host_fp32, h->stream));
            else
                GPE_CUDA_TRY(launch_pack(prec, h->idev, i, in.nx, in.ny, in.nz, h->ns, src, field_buf(h, f), 1, 1.0,
                                         h->stream));
            h->launches++;
        }
        if (arr) {
            const size_t b = vals * h->esize;
            const void *src = mapped[3 * k + 2];
            if (src) h->mapped_transfers++;
            else {
                if ((st = copy_in(stage, potential[k], b)) != GPE_OK) return st;
                src = stage;
                stage += slot_bytes(b);
            }
            GPE_CUDA_TRY(launch_pack(prec, h->idev, i, in.nx, in.ny, in.nz, h->ns, src, h->vpot, 0, in.dt, h->stream));
            GPE_CUDA_TRY(launch_potential_base(prec, h->idev, i, in.nx, in.ny, in.nz, h->ns, h->vpot, h->vbase,
                                               h->stream));
            h->launches += 2;
        }
    }
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->imag_ready = false;
    return GPE_OK;
}

gpe_status gpe_upload_many(gpe_handle h, int32_t count, const int32_t *instances, const void *const *even,
                           const void *const *odd, const void *const *potential)
{
    GPE_GUARD(gpe_upload_many_impl(h, count, instances, even, odd, potential));
}

static gpe_status gpe_download_many_impl(gpe_handle h, int32_t count, const int32_t *instances, void *const *even,
                                         void *const *odd)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (count < 0 || (count > 0 && !instances))
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_download_many: bad count or null array");
    // Buffers in mapped page-locked memory receive the conversion's output in
    // place; the others go through staging and a copy.
    std::vector<void *> mapped(size_t(count) * 2, nullptr);
    size_t total = 0;
    for (int k = 0; k < count; k++) {
        const int i = instances[k];
        if (i < 0 || i >= h->cfg.num_instances)
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_download_many: bad instance");
        const gpe_instance &in = h->inst[i];
        const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
        void *dsts[2] = {even ? even[k] : nullptr, odd ? odd[k] : nullptr};
        for (int f = 0; f < 2; f++) {
            if (!dsts[f]) continue;
            mapped[2 * k + f] = mapped_host_range(dsts[f], vals * 2 * h->hsize, 2 * h->hsize, h->cfg.device);
            if (!mapped[2 * k + f]) total += slot_bytes(vals * 2 * h->hsize);
        }
    }
    st = sync_and_check(h);
    if (st != GPE_OK) return st;
    if (total == 0) {  // every buffer in mapped memory: one in-place launch
        std::vector<std::tuple<const void *, int, int>> items;
        for (int k = 0; k < count; k++)
            for (int f = 0; f < 2; f++)
                if (mapped[2 * k + f]) items.emplace_back(mapped[2 * k + f], instances[k], f);
        if (!items.empty() && (st = run_xfer_batch(h, false, items)) != GPE_OK) return st;
        GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
        return GPE_OK;
    }
    st = ensure_batch_staging(h, std::max<size_t>(total, 256));
    if (st == GPE_OK) st = ensure_xfer(h, size_t(2) * count);
    if (st != GPE_OK) return st;
    char *stage = (char *)h->batch_staging;
    // Conversions on the handle's stream; each copy waits for its conversion on
    // the copy stream, so copies overlap later conversions.
    size_t ev = 0;
    for (int k = 0; k < count; k++) {
        const int i = instances[k];
        const gpe_instance &in = h->inst[i];
        const size_t vals = size_t(in.nx) * in.ny * in.nz * h->ns;
        void *dsts[2] = {even ? even[k] : nullptr, odd ? odd[k] : nullptr};
        for (int f = 0; f < 2; f++) {
            if (!dsts[f]) continue;
            const size_t b = vals * 2 * h->hsize;
            void *out = mapped[2 * k + f] ? mapped[2 * k + f] : stage;
            if (mapped[2 * k + f]) h->mapped_transfers++;
            if (h->comp)
                GPE_CUDA_TRY(launch_unpack_join(h->idev, i, in.nx, in.ny, in.nz, h->ns, field_buf(h, f), h->lo[f], out,
                                                h->host_fp32, h->stream));
            else
                GPE_CUDA_TRY(launch_unpack(h->cfg.precision, h->idev, i, in.nx, in.ny, in.nz, h->ns, field_buf(h, f),
                                           out, nullptr, h->stream));
            h->launches++;
            if (mapped[2 * k + f]) continue;
            GPE_CUDA_TRY(cudaEventRecord(h->xfer_events[ev], h->stream));
            GPE_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->xfer_events[ev++], 0));
            GPE_CUDA_TRY(cudaMemcpyAsync(dsts[f], stage, b, cudaMemcpyDeviceToHost, h->copy_stream));
            stage += slot_bytes(b);
        }
    }
    GPE_CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GPE_OK;
}

gpe_status gpe_download_many(gpe_handle h, int32_t count, const int32_t *instances, void *const *even,
                             void *const *odd)
{
    GPE_GUARD(gpe_download_many_impl(h, count, instances, even, odd));
}

static gpe_status gpe_step_impl(gpe_handle h, int64_t steps)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (steps < 0) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_step: negative step count");
    if (steps == 0) return GPE_OK;
    if (!h->zlinks.empty()) {  // halos of both fields as uploaded
        st = enqueue_halo(h, 0);
        if (st == GPE_OK) st = enqueue_halo(h, 1);
        if (st != GPE_OK) return st;
    }
    if (h->cfg.mode == GPE_IMAGINARY_TIME) {
        st = imag_prepare(h);
        if (st != GPE_OK) return st;
    }
    st = run_steps(h, steps);
    if (st != GPE_OK) return st;
    if (h->cfg.mode == GPE_IMAGINARY_TIME) {
        st = imag_normalise(h, !h->fused);
        if (st != GPE_OK) return st;
    }
    return GPE_OK;
}

gpe_status gpe_step(gpe_handle h, int64_t steps)
{
    GPE_GUARD(gpe_step_impl(h, steps));
}

static gpe_status gpe_synchronize_impl(gpe_handle h)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    return sync_and_check(h);
}

gpe_status gpe_synchronize(gpe_handle h)
{
    GPE_GUARD(gpe_synchronize_impl(h));
}

namespace {

// The observables sums of every instance's field `field` into h->obs_sums: one
// launch over all instances, then one CTA per instance folds its rows (the same
// sums as one launch per instance).
gpe_status enqueue_observables_all(gpe_handle h, int field)
{
    GPE_CUDA_TRY(launch_observables_batch(h->cfg.lattice, h->cfg.precision, h->cfg.potential, h->idev, h->obs_cta_inst,
                                          h->obs_cta_begin, h->obs_total_ctas, field_buf(h, field), h->vpot,
                                          h->obs_batch_partials, h->stream));
    GPE_CUDA_TRY(launch_reduce_partials_batch(h->obs_batch_partials, h->obs_cta_begin, h->cfg.num_instances,
                                              h->obs_sums, h->stream));
    h->launches += 2;
    return GPE_OK;
}

// gpe_observables records from the six sums per instance.
gpe_status observables_from_sums(gpe_handle h, const std::vector<double> &sums, gpe_observables *out,
                                 const char *where)
{
    bool all_finite = true;
    for (int i = 0; i < h->cfg.num_instances; i++) {
        const double vol = h->idev_host[i].vol;
        gpe_observables &o = out[i];
        o.norm = vol * sums[6 * i + 0];
        o.kinetic = vol * sums[6 * i + 1];
        o.potential = vol * sums[6 * i + 2];
        o.interaction = vol * sums[6 * i + 3];
        o.energy = o.kinetic + o.potential + o.interaction;
        o.mu = (o.kinetic + o.potential + 2.0 * o.interaction) / o.norm;
        o.finite = std::isfinite(o.norm) && std::isfinite(o.energy) && std::isfinite(o.mu);
        o.pad_ = 0;
        all_finite = all_finite && o.finite;
    }
    if (!all_finite) return fail(GPE_ERR_NOT_FINITE, std::string(where) + ": NaN or Inf in the field");
    return GPE_OK;
}

}  // namespace

static gpe_status gpe_observables_get_impl(gpe_handle h, int32_t field, gpe_observables *out)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (!out || (field != 0 && field != 1)) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_observables_get: bad arguments");
    if ((st = enqueue_observables_all(h, field)) != GPE_OK) return st;
    std::vector<double> sums(6 * h->cfg.num_instances);
    GPE_CUDA_TRY(cudaMemcpyAsync(sums.data(), h->obs_sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost,
                                 h->stream));
    st = sync_and_check(h);
    if (st != GPE_OK) return st;
    return observables_from_sums(h, sums, out, "gpe_observables_get");
}

gpe_status gpe_observables_get(gpe_handle h, int32_t field, gpe_observables *out)
{
    GPE_GUARD(gpe_observables_get_impl(h, field, out));
}

namespace {

// On every way out of a round trip: the full item range for later step
// launches again, and no copy still touching the caller's buffers.
struct RoundTripExit {
    gpe_handle h;
    ~RoundTripExit()
    {
        h->run_first = h->run_count = 0;
        if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
        if (h->down_stream) cudaStreamSynchronize(h->down_stream);
    }
};

}  // namespace

static gpe_status gpe_round_trip_impl(gpe_handle h, const void *const *even_in, const void *const *odd_in,
                                      int64_t steps, void *const *even_out, void *const *odd_out,
                                      gpe_observables *obs)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    const int n = h->cfg.num_instances;
    const bool real = h->cfg.mode == GPE_REAL_TIME;
    if (steps < 0) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_round_trip: negative step count");
    if (!even_in || (real && !odd_in)) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_round_trip: null input array");
    for (int i = 0; i < n; i++)
        if (!even_in[i] || (real && !odd_in[i]))
            return fail(GPE_ERR_INVALID_ARGUMENT,
                        "gpe_round_trip: input field of instance " + std::to_string(i) + " is null");
    // Instance groups only where a launch can cover a subset of the instances:
    // the fused half-step kernels in real time, no slabs.
    const bool split = real && h->fused && !h->two_step && !h->persistent && h->zlinks.empty() && steps > 0 &&
                       int(h->item_order.size()) == n && n > 1;
    // Groups and their rolling schedule (gpe_round_trip_plan.h).  R: a value's
    // upload (four host elements at about 200 GB/s over the host link) against
    // one step of it in HBM (B bytes per value-step at about 6 TB/s).
    std::vector<long long> values(n);
    for (int i = 0; i < n; i++) values[i] = (long long)h->inst[i].nx * h->inst[i].ny * h->inst[i].nz * h->ns;
    const double B = h->comp ? 56.0 : (h->cfg.precision == GPE_FP64 ? 96.0 : 48.0);
    const RoundTripPlan plan =
        plan_round_trip(values, h->item_order, split, steps, 4.0 * double(h->hsize) / 200.0 * 6000.0 / B);
    const std::vector<std::vector<int>> &groups = plan.groups;
    const std::vector<long long> &join = plan.join;
    const int G = int(groups.size());
    // One staging slot per (instance, field), holding the upload and then the download.
    std::vector<size_t> off(2 * size_t(n));
    size_t total = 0;
    for (int i = 0; i < n; i++) {
        const gpe_instance &in = h->inst[i];
        const size_t b = size_t(in.nx) * in.ny * in.nz * h->ns * 2 * h->hsize;
        for (int f = 0; f < 2; f++) {
            off[2 * i + f] = total;
            const bool in_used = f == 0 || (odd_in && odd_in[i]);
            const bool out_used = f == 0 ? (even_out && even_out[i]) : (odd_out && odd_out[i]);
            if (in_used || out_used) total += slot_bytes(b);
        }
    }
    st = ensure_batch_staging(h, std::max<size_t>(total, 256));
    if (st == GPE_OK) st = ensure_xfer(h, size_t(2 * G + 1));
    if (st != GPE_OK) return st;
    if (!h->down_stream) GPE_CUDA_TRY(cudaStreamCreateWithFlags(&h->down_stream, cudaStreamNonBlocking));
    RoundTripExit guard{h};
    char *stage = (char *)h->batch_staging;
    cudaEvent_t *ev = h->xfer_events.data();  // [0] start, [1..G] group uploaded, [G+1..2G] group converted
    auto bytes_of = [&](int i) {
        const gpe_instance &in = h->inst[i];
        return size_t(in.nx) * in.ny * in.nz * h->ns * 2 * h->hsize;
    };
    // Layout conversions between the staging slots and the fields: one launch
    // per group and direction (the batched transfer kernel, reading or writing
    // the slots instead of host memory).  Every launch's segment table goes to
    // the device here, before any work is queued.
    std::vector<XferSeg> &segs = h->xfer_segs_host;
    segs.clear();
    std::vector<int> seg_at(2 * G), seg_n(2 * G), seg_ctas(2 * G);
    for (int g = 0; g < G; g++)
        for (int dir = 0; dir < 2; dir++) {
            const int L = 2 * g + dir;
            seg_at[L] = int(segs.size());
            int cta = 0;
            for (int i : groups[g])
                for (int f = 0; f < 2; f++) {
                    const bool used = dir == 0 ? (f == 0 || (odd_in && odd_in[i]))
                                               : (f == 0 ? even_out && even_out[i] : odd_out && odd_out[i]);
                    if (!used) continue;
                    const long long vals = (long long)h->inst[i].nx * h->inst[i].ny * h->inst[i].nz * h->ns;
                    segs.push_back({stage + off[2 * i + f], i, f, cta, 0});
                    cta += int((vals + kXferValuesPerCta - 1) / kXferValuesPerCta);
                }
            seg_n[L] = int(segs.size()) - seg_at[L];
            seg_ctas[L] = cta;
            segs.push_back({nullptr, 0, 0, cta, 0});
        }
    if (segs.size() > h->xfer_segs_cap) {
        cudaFree(h->xfer_segs);
        h->xfer_segs = nullptr;
        h->xfer_segs_cap = 0;
        GPE_CUDA_TRY(cudaMalloc(&h->xfer_segs, sizeof(XferSeg) * segs.size()));
        h->xfer_segs_cap = segs.size();
    }
    GPE_CUDA_TRY(cudaMemcpyAsync(h->xfer_segs, segs.data(), sizeof(XferSeg) * segs.size(), cudaMemcpyHostToDevice,
                                 h->stream));
    auto convert = [&](int g, bool up) -> gpe_status {
        const int L = 2 * g + (up ? 0 : 1);
        if (seg_n[L] == 0) return GPE_OK;
        GPE_CUDA_TRY(launch_xfer_batch(h->cfg.precision, h->comp, h->host_fp32, up, h->idev, h->xfer_segs + seg_at[L],
                                       seg_n[L], seg_ctas[L], field_buf(h, 0), field_buf(h, 1), h->lo[0], h->lo[1],
                                       h->stream));
        h->launches++;
        return GPE_OK;
    };
    // Group g's copies up, on the copy stream, then its event ev[1 + g].
    auto upload = [&](int g) -> gpe_status {
        for (int i : groups[g]) {
            const void *src[2] = {even_in[i], odd_in ? odd_in[i] : nullptr};
            for (int f = 0; f < 2; f++)
                if (src[f])
                    GPE_CUDA_TRY(cudaMemcpyAsync(stage + off[2 * i + f], src[f], bytes_of(i), cudaMemcpyHostToDevice,
                                                 h->copy_stream));
        }
        GPE_CUDA_TRY(cudaEventRecord(ev[1 + g], h->copy_stream));
        return GPE_OK;
    };
    // Group g joins: wait for its copies, convert them into the fields.
    std::vector<bool> has_out(G, false);
    auto join_group = [&](int g) -> gpe_status {
        GPE_CUDA_TRY(cudaStreamWaitEvent(h->stream, ev[1 + g], 0));
        gpe_status s2 = convert(g, true);
        h->imag_ready = false;
        return s2;
    };
    // Group g leaves: convert its fields into its slots, then ev[G + 1 + g].
    auto leave_group = [&](int g) -> gpe_status {
        has_out[g] = seg_n[2 * g + 1] > 0;
        gpe_status s2 = convert(g, false);
        if (s2 != GPE_OK) return s2;
        if (has_out[g]) GPE_CUDA_TRY(cudaEventRecord(ev[G + 1 + g], h->stream));
        return GPE_OK;
    };
    // Group g's copies down, on the down stream, after its conversions.
    auto download = [&](int g) -> gpe_status {
        if (!has_out[g]) return GPE_OK;
        GPE_CUDA_TRY(cudaStreamWaitEvent(h->down_stream, ev[G + 1 + g], 0));
        for (int i : groups[g]) {
            void *dst[2] = {even_out ? even_out[i] : nullptr, odd_out ? odd_out[i] : nullptr};
            for (int f = 0; f < 2; f++)
                if (dst[f])
                    GPE_CUDA_TRY(cudaMemcpyAsync(dst[f], stage + off[2 * i + f], bytes_of(i), cudaMemcpyDeviceToHost,
                                                 h->down_stream));
        }
        return GPE_OK;
    };
    // The rounds: every active group advances one leapfrog step per round, in
    // launches over the active groups' items (consecutive in the item order);
    // groups join as their uploads should have landed and leave after K steps,
    // so most launches cover several groups.  A group's first launch waits for
    // its copies, so an estimate off either way only costs overlap.
    // Host order: U0, then every copy is queued after the compute it overlaps
    // (U(g+1) after group g's first piece), so the overlap holds even where the
    // runtime makes a copy call wait on the host.  Downloads queue once every
    // upload is queued and wait for the last one, so an output buffer may be any
    // instance's input buffer; they go in before the observables' read-back,
    // which waits.
    GPE_CUDA_TRY(cudaEventRecord(ev[0], h->stream));  // earlier work on the handle's stream first
    GPE_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, ev[0], 0));
    GPE_CUDA_TRY(cudaStreamWaitEvent(h->down_stream, ev[0], 0));
    if ((st = upload(0)) != GPE_OK) return st;
    int uploaded = 1, left = 0, next_down = 0;
    if (G == 1) GPE_CUDA_TRY(cudaStreamWaitEvent(h->down_stream, ev[G], 0));
    for (const RoundTripPiece &piece : plan.pieces) {
        const long long r0 = piece.r0, r1 = piece.r1;
        const int lo = piece.lo, hi = piece.hi;
        for (int g = 0; g < G; g++)
            if (join[g] == r0 && (st = join_group(g)) != GPE_OK) return st;
        if (lo <= hi) {
            if (split) {
                h->run_first = h->item_first[groups[lo][0]];
                h->run_count = 0;
                for (int g = lo; g <= hi; g++)
                    for (int i : groups[g]) {
                        h->run_first = std::min(h->run_first, h->item_first[i]);
                        h->run_count += h->item_count[i];
                    }
                st = run_steps(h, r1 - r0);
            } else {
                st = gpe_step_impl(h, r1 - r0);
            }
            if (st != GPE_OK) return st;
        }
        for (int g = 0; g < G; g++)
            if (join[g] + steps == r1 && (st = leave_group(g)) != GPE_OK) return st;
        while (left < G && join[left] + steps <= r1) left++;
        while (uploaded < G && join[uploaded - 1] <= r0) {
            if ((st = upload(uploaded++)) != GPE_OK) return st;
            if (uploaded == G) GPE_CUDA_TRY(cudaStreamWaitEvent(h->down_stream, ev[G], 0));
        }
        if (uploaded == G)
            while (next_down < left)
                if ((st = download(next_down++)) != GPE_OK) return st;
    }
    while (uploaded < G) {
        if ((st = upload(uploaded++)) != GPE_OK) return st;
        if (uploaded == G) GPE_CUDA_TRY(cudaStreamWaitEvent(h->down_stream, ev[G], 0));
    }
    if (steps == 0)  // no rounds: convert and return the fields as uploaded
        for (int g = 0; g < G; g++)
            if ((st = join_group(g)) != GPE_OK || (st = leave_group(g)) != GPE_OK) return st;
    while (next_down < G)
        if ((st = download(next_down++)) != GPE_OK) return st;
    // The observables run while the last group's fields travel down.
    std::vector<double> sums;
    if (obs) {
        if ((st = enqueue_observables_all(h, 0)) != GPE_OK) return st;
        sums.resize(6 * size_t(n));
        GPE_CUDA_TRY(cudaMemcpyAsync(sums.data(), h->obs_sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost,
                                     h->stream));
    }
    GPE_CUDA_TRY(cudaStreamSynchronize(h->down_stream));
    GPE_CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
    st = sync_and_check(h);
    if (st != GPE_OK) return st;
    return obs ? observables_from_sums(h, sums, obs, "gpe_round_trip") : GPE_OK;
}

gpe_status gpe_round_trip(gpe_handle h, const void *const *even_in, const void *const *odd_in, int64_t steps,
                          void *const *even_out, void *const *odd_out, gpe_observables *obs)
{
    GPE_GUARD(gpe_round_trip_impl(h, even_in, odd_in, steps, even_out, odd_out, obs));
}

static gpe_status gpe_observables_get_impl(gpe_handle h, int32_t field, gpe_observables *out);

static gpe_status gpe_imaginary_time_impl(gpe_handle h, int64_t max_steps, double tol, int64_t *steps_done, int32_t *converged,
                                          double *mu_out)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (h->cfg.mode != GPE_IMAGINARY_TIME)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_imaginary_time: handle is not in imaginary-time mode");
    if (max_steps < 0 || !(tol >= 0.0)) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_imaginary_time: bad arguments");
    // FP64: the per-step test |mu_k - mu_(k-1)| < tol on the device, as the
    // reductions fused into each step compute mu.  FP32: a per-step difference
    // of mu taken from FP32 values is not resolvable at tol (a step can change
    // no stored value, or change it by less than the sums' rounding), so after
    // every chunk of G steps mu of the normalised field is taken from the FP64
    // observables, and the run has converged when |mu_k - mu_(k-W)| < W * tol
    // over the last W = kWindowChunks * G steps: the mean change per step over
    // that window is below tol.  A window of one chunk stopped a 128^3
    // random-phase start on a slow plateau, 1e-4 above the FP64 run's mu.
    const bool windowed = h->cfg.precision != GPE_FP64;
    h->tol = windowed ? 0.0 : tol;
    st = imag_prepare(h);
    if (st != GPE_OK) return st;
    const long long G = h->cfg.graph_steps == 0 ? 100 : (h->cfg.graph_steps < 0 ? 100 : h->cfg.graph_steps);
    long long done = 0;
    bool all = false;
    const int n_inst = h->cfg.num_instances;
    std::vector<ImagScalars> sc(n_inst);
    std::vector<gpe_observables> obs(n_inst);
    constexpr int kWindowChunks = 10;
    std::vector<double> mu(n_inst, 0.0);
    std::vector<std::vector<double>> hist;  // mu after each of the last kWindowChunks full chunks
    while (done < max_steps) {
        const long long n = std::min<long long>(G, max_steps - done);
        st = run_steps(h, n);
        if (st != GPE_OK) return st;
        done += n;
        st = imag_normalise(h, !h->fused);
        if (st != GPE_OK) return st;
        if (windowed) {
            st = gpe_observables_get_impl(h, 0, obs.data());
            if (st != GPE_OK) return st;
            for (int i = 0; i < n_inst; i++) mu[i] = obs[i].mu;
            all = n == G && int(hist.size()) == kWindowChunks;
            for (int i = 0; all && i < n_inst; i++)
                all = std::fabs(mu[i] - hist.front()[i]) < double(kWindowChunks * G) * tol;
            if (n == G) {
                hist.push_back(mu);
                if (int(hist.size()) > kWindowChunks) hist.erase(hist.begin());
            }
        } else {
            GPE_CUDA_TRY(cudaMemcpyAsync(sc.data(), h->imag, sizeof(ImagScalars) * sc.size(), cudaMemcpyDeviceToHost,
                                         h->stream));
            st = sync_and_check(h);
            if (st != GPE_OK) return st;
            all = true;
            for (int i = 0; i < n_inst; i++) {
                all = all && (sc[i].conv_step >= 0);
                mu[i] = sc[i].mu;
            }
        }
        if (all) break;
    }
    if (steps_done) *steps_done = done;
    if (converged) *converged = all ? 1 : 0;
    if (mu_out)
        for (int i = 0; i < n_inst; i++) mu_out[i] = mu[i];
    return GPE_OK;
}

gpe_status gpe_imaginary_time(gpe_handle h, int64_t max_steps, double tol, int64_t *steps_done, int32_t *converged,
                              double *mu_out)
{
    GPE_GUARD(gpe_imaginary_time_impl(h, max_steps, tol, steps_done, converged, mu_out));
}

static gpe_status gpe_time_steps_impl(gpe_handle h, int64_t steps, float *ms)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (!ms || steps < 0) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_time_steps: bad arguments");
    cudaEvent_t a = nullptr, b = nullptr;
    GPE_CUDA_TRY(cudaEventCreate(&a));
    cudaError_t e = cudaEventCreate(&b);
    if (e != cudaSuccess) {
        cudaEventDestroy(a);
        return cuda_fail(e, "cudaEventCreate");
    }
    e = cudaEventRecord(a, h->stream);
    if (e == cudaSuccess) st = gpe_step(h, steps);
    if (e == cudaSuccess && st == GPE_OK) e = cudaEventRecord(b, h->stream);
    if (e == cudaSuccess && st == GPE_OK) e = cudaEventSynchronize(b);
    if (e == cudaSuccess && st == GPE_OK) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != GPE_OK) return st;
    if (e != cudaSuccess) return cuda_fail(e, "gpe_time_steps");
    return sync_and_check(h);
}

gpe_status gpe_time_steps(gpe_handle h, int64_t steps, float *ms)
{
    GPE_GUARD(gpe_time_steps_impl(h, steps, ms));
}

static gpe_status gpe_debug_inject_impl(gpe_handle h, int32_t plane)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (!h->fused) return fail(GPE_ERR_UNSUPPORTED, "gpe_debug_inject: only the fused kernel has device waits");
    h->inject = plane < 0 ? -1 : plane;
    // launches already captured into graphs carry the old value
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return GPE_OK;
}

gpe_status gpe_debug_inject(gpe_handle h, int32_t plane)
{
    GPE_GUARD(gpe_debug_inject_impl(h, plane));
}

static gpe_status gpe_volume_map_impl(gpe_handle h, int32_t instance, int32_t field, double unit, int32_t reference_sum,
                                      uint16_t *out)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (instance < 0 || instance >= h->cfg.num_instances || (field != 0 && field != 1) || !out)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_volume_map: bad arguments");
    const gpe_instance &in = h->inst[instance];
    const long long total = (long long)(in.nx + 2) * (in.ny + 2) * (in.nz + 2);
    GPE_CUDA_TRY(launch_volume(h->cfg.precision, h->idev, instance, field_buf(h, field), unit, reference_sum ? 1 : 0,
                               (uint16_t *)h->staging, total, h->stream));
    h->launches++;
    GPE_CUDA_TRY(cudaMemcpyAsync(out, h->staging, size_t(total) * 2, cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

gpe_status gpe_volume_map(gpe_handle h, int32_t instance, int32_t field, double unit, int32_t reference_sum,
                          uint16_t *out)
{
    GPE_GUARD(gpe_volume_map_impl(h, instance, field, unit, reference_sum, out));
}

static gpe_status gpe_slice_rgb_impl(gpe_handle h, int32_t instance, int32_t field, int32_t z_padded, int32_t slot, double gain,
                                     uint8_t *out)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (instance < 0 || instance >= h->cfg.num_instances || (field != 0 && field != 1) || !out || slot < 0 ||
        slot >= h->ns)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_slice_rgb: bad arguments");
    const gpe_instance &in = h->inst[instance];
    const int total = (in.nx + 2) * (in.ny + 2);
    GPE_CUDA_TRY(launch_slice(h->cfg.precision, h->idev, instance, field_buf(h, field), z_padded, slot, gain,
                              (uint8_t *)h->staging, total, h->stream));
    h->launches++;
    GPE_CUDA_TRY(cudaMemcpyAsync(out, h->staging, size_t(total) * 3, cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

gpe_status gpe_slice_rgb(gpe_handle h, int32_t instance, int32_t field, int32_t z_padded, int32_t slot, double gain,
                         uint8_t *out)
{
    GPE_GUARD(gpe_slice_rgb_impl(h, instance, field, z_padded, slot, gain, out));
}

static gpe_status gpe_link_z_impl(gpe_handle h, int32_t lower, int32_t upper)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (h->cfg.mode != GPE_REAL_TIME)
        return fail(GPE_ERR_UNSUPPORTED, "gpe_link_z: slabs are supported in real time (imaginary time "
                                         "normalises each instance on its own)");
    if (h->two_step || h->persistent)
        return fail(GPE_ERR_UNSUPPORTED, "gpe_link_z: slabs exchange halos between half-steps; use a kernel "
                                         "variant that advances a half-step per launch");
    const int n = h->cfg.num_instances;
    if (lower < 0 || lower >= n || upper < 0 || upper >= n || lower == upper)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_link_z: bad instance indices");
    const InstDev &lo = h->idev_host[lower], &up = h->idev_host[upper];
    if (lo.nx != up.nx || lo.ny != up.ny || lo.px != up.px)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_link_z: linked slabs need the same nx and ny");
    for (auto &lk : h->zlinks)
        if (lk.first == lower || lk.second == upper)
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_link_z: a slab has one neighbour per side");
    h->zlinks.push_back({lower, upper});
    h->slots_from_above = h->slots_from_below = 0;
    for (int s = 0; s < h->lat.slots; s++)
        for (int k = 0; k < h->lat.neighbours; k++) {
            const int dz = h->lat.entry[s][k][2], sl = h->lat.entry[s][k][3];
            if (dz > 0) h->slots_from_above |= 1u << sl;
            if (dz < 0) h->slots_from_below |= 1u << sl;
        }
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second);  // captured steps lack the new copies
    h->graphs.clear();
    return GPE_OK;
}

gpe_status gpe_link_z(gpe_handle h, int32_t lower, int32_t upper)
{
    GPE_GUARD(gpe_link_z_impl(h, lower, upper));
}

static gpe_status gpe_set_host_precision_impl(gpe_handle h, int32_t precision)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (h->comp) {
        if (precision != GPE_FP64 && precision != GPE_FP32)
            return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_set_host_precision: GPE_FP32C exchanges fields as GPE_FP64 "
                                                  "or GPE_FP32");
        h->host_fp32 = precision == GPE_FP32;
        h->hsize = h->host_fp32 ? 4 : 8;
        return GPE_OK;
    }
    if (precision != h->cfg.precision)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_set_host_precision: this handle exchanges fields in its own "
                                              "precision");
    return GPE_OK;
}

gpe_status gpe_set_host_precision(gpe_handle h, int32_t precision)
{
    GPE_GUARD(gpe_set_host_precision_impl(h, precision));
}

int32_t gpe_variant_count(void) { return fused_tile_count(); }

int32_t gpe_variant_half_steps(int32_t variant)
{
    return (variant >= 0 && variant < fused_tile_count()) ? fused_half_steps(variant) : 0;
}

int32_t gpe_variant_kind(int32_t variant)
{
    return (variant >= 0 && variant < fused_tile_count()) ? fused_variant_kind(variant) : -1;
}

static gpe_status gpe_variant_describe_impl(int32_t variant, int32_t *tile_x, int32_t *tile_y, int32_t *stages,
                                            int32_t *min_blocks)
{
    if (variant < 0 || variant >= fused_tile_count())
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_variant_describe: no such variant");
    int tx, ty, stg, mb;
    fused_variant(variant, &tx, &ty, &stg, &mb);
    if (tile_x) *tile_x = tx;
    if (tile_y) *tile_y = ty;
    if (stages) *stages = stg;
    if (min_blocks) *min_blocks = mb;
    return GPE_OK;
}

gpe_status gpe_variant_describe(int32_t variant, int32_t *tile_x, int32_t *tile_y, int32_t *stages,
                                int32_t *min_blocks)
{
    GPE_GUARD(gpe_variant_describe_impl(variant, tile_x, tile_y, stages, min_blocks));
}

int64_t gpe_launch_count(gpe_handle h) { return h ? h->launches : 0; }

int64_t gpe_mapped_transfers(gpe_handle h) { return h ? h->mapped_transfers : 0; }

void *gpe_stream(gpe_handle h) { return h ? (void *)h->stream : nullptr; }

}  // extern "C"

namespace gpe {

gpe_status upload_device_fields(gpe_handle h, int32_t instance, const void *even, const void *odd,
                                const void *potential)
{
    gpe_status st = check_handle(h);
    if (st != GPE_OK) return st;
    if (instance < 0 || instance >= h->cfg.num_instances)
        return fail(GPE_ERR_INVALID_ARGUMENT, "upload_device_fields: bad instance");
    if (h->comp) return fail(GPE_ERR_UNSUPPORTED, "upload_device_fields: not for GPE_FP32C");
    if (!even || (h->cfg.mode == GPE_REAL_TIME && !odd) || (h->cfg.potential == GPE_POTENTIAL_ARRAY && !potential))
        return fail(GPE_ERR_INVALID_ARGUMENT, "upload_device_fields: missing field or potential");
    const gpe_instance &in = h->inst[instance];
    const int prec = h->cfg.precision;
    const void *srcs[2] = {even, odd};
    for (int f = 0; f < 2; f++) {
        if (!srcs[f]) continue;
        GPE_CUDA_TRY(launch_pack(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, srcs[f], field_buf(h, f), 1,
                                 1.0, h->stream));
        h->launches++;
    }
    if (h->cfg.potential == GPE_POTENTIAL_ARRAY) {
        GPE_CUDA_TRY(launch_pack(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, potential, h->vpot, 0, in.dt,
                                 h->stream));
        GPE_CUDA_TRY(launch_potential_base(prec, h->idev, instance, in.nx, in.ny, in.nz, h->ns, h->vpot, h->vbase,
                                           h->stream));
        h->launches += 2;
    }
    GPE_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->imag_ready = false;
    return GPE_OK;
}

}  // namespace gpe
