// gpe_noalloc.cu - observables of one condensate held in caller-owned device
// memory, computed without allocating memory.
//
// Who needs it: callers that cannot call cudaMalloc.  Typical cases are an
// application whose device memory is entirely handed out by its own pool (or a
// framework's), so that any allocation outside that pool is forbidden or would
// fail, and code on a latency-critical path where cudaMalloc/cudaFree - which can
// synchronise the whole device - must not run.  gpe_observables_get needs a
// handle, and a handle allocates its arenas at gpe_create; this entry point
// needs neither.
//
// Scratch: the per-CTA partial sums live in the file-scope device array below
// (kRows rows of 6 doubles plus one row for the final sums, 384 KiB plus 48
// bytes).  Every GPU that loads this library holds it until the process exits.
// Each CTA sums kPerRow values, so one call accepts at most kRows * kPerRow
// values; larger inputs are rejected with GPE_ERR_TOO_LARGE.  Every call
// rewrites every row it later reads, so nothing has to be cleared between calls;
// the array keeps the last call's contents.  All calls share the one array:
// calls whose kernels overlap on the GPU (different streams, or host threads
// racing on one device) corrupt each other's sums - serialise them.
//
// Set-up: host code cannot use the array's name as a device address, so the
// first call on each device (with that device current) looks the address up
// with cudaGetSymbolAddress and caches it; that first call should therefore be
// made before any stream capture begins.  The cache is keyed on the device's
// current CUDA context by its process-unique id (cuCtxGetId), so after a
// cudaDeviceReset, or any other change of context, the next call looks the
// address up again instead of using one from a destroyed context.  The stencil
// tables are computed when the library is loaded.

#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "gpe_internal.h"

namespace gpe {
namespace {

constexpr int kRows = GPE_NOALLOC_MAX_ROWS;
constexpr int kThreads = 256;
constexpr int kPerThread = GPE_NOALLOC_VALUES_PER_ROW / kThreads;
constexpr int kPerRow = GPE_NOALLOC_VALUES_PER_ROW;
constexpr int kMaxDevices = 64;

// rows [0, kRows): one row of 6 partial sums per CTA; row kRows: the final sums
static __device__ __align__(256) double g_noalloc_scratch[(kRows + 1) * 6];

// Host-side cache of the array's device address, per device ordinal, valid for
// the context whose id it records.
struct ScratchAddr {
    unsigned long long ctx_id = 0;
    double *ptr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mutex;

// cuCtxGetCurrent and cuCtxGetId through the runtime's driver entry point (the
// library links only the CUDA runtime); looked up once.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
struct CtxFns {
    CtxGetCurrentFn current = nullptr;
    CtxGetIdFn id = nullptr;
    CtxFns()
    {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            current = (CtxGetCurrentFn)fn;
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            id = (CtxGetIdFn)fn;
    }
};

// Id of the calling thread's current context; 0 if there is none or it cannot
// be told (then the address is looked up on every call).
unsigned long long current_context_id()
{
    static const CtxFns fns;
    if (!fns.current || !fns.id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (fns.current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (fns.id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Stencil of each lattice, packed for the kernel and passed by value.
struct NoallocStencil {
    int slots, neighbours;
    int entry[12 * 14];  // (dx+1) | (dy+1)<<2 | (dz+1)<<4 | slot<<6 | class<<10
    double cls_weight[2];
    double cell_volume;
    double block_width;
    double position[12][3];
};

struct StencilCache {
    NoallocStencil s[2];
    bool ok = false;
    StencilCache()
    {
        ok = true;
        for (int lat = 0; lat < 2; lat++) {
            gpe_lattice_info info;
            if (build_lattice(gpe_lattice(lat), &info) != GPE_OK) {
                ok = false;
                continue;
            }
            NoallocStencil &t = s[lat];
            t.slots = info.slots;
            t.neighbours = info.neighbours;
            for (int sl = 0; sl < info.slots; sl++)
                for (int k = 0; k < info.neighbours; k++) {
                    const int *e = info.entry[sl][k];
                    t.entry[sl * info.neighbours + k] =
                        (e[0] + 1) | ((e[1] + 1) << 2) | ((e[2] + 1) << 4) | (e[3] << 6) | (e[4] << 10);
                }
            t.cls_weight[0] = info.class_weight[0];
            t.cls_weight[1] = info.classes > 1 ? info.class_weight[1] : 0.0;
            t.cell_volume = info.cell_volume;
            t.block_width = info.block_width;
            for (int sl = 0; sl < info.slots; sl++)
                for (int c = 0; c < 3; c++) t.position[sl][c] = info.position[sl][c];
        }
    }
};
const StencilCache g_stencils;  // built at library load, not inside a call

struct NoallocGrid {
    int nx, ny, nz;
    double w[2];      // class weights / block_scale^2
    double g;
    double bs, origin[3], trap[3];
};

// Same sums as observables_kernel, for the reference's block order
// (((z*ny)+y)*nx+x)*slots+s with psi = 0 outside the grid: |psi|^2,
// Re(conj(psi)(-1/2 Lap psi)), V|psi|^2, g/2 |psi|^4.  V comes from `vpot`
// (unscaled, same order) or, when it is null, from the harmonic trap.
template <typename T>
__global__ void __launch_bounds__(kThreads) noalloc_observables_kernel(const NoallocStencil st, const NoallocGrid gr,
                                                                     const T *__restrict__ f,
                                                                     const T *__restrict__ vpot, long long total)
{
    double *rows = g_noalloc_scratch;
    const int ns = st.slots, nb = st.neighbours;
    int n0 = 0;
    for (int k = 0; k < nb; k++) n0 += ((st.entry[k] >> 10) & 3) == 0;
    const double wsum = n0 * gr.w[0] + (nb - n0) * gr.w[1];
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0, s2 = 0, c2 = 0, s3 = 0, c3 = 0;
    auto kahan = [](double &s, double &c, double v) {
        const double y = v - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    };
    const long long first = (long long)blockIdx.x * kPerRow;
    for (int j = 0; j < kPerThread; j++) {
        const long long v = first + j * kThreads + threadIdx.x;
        if (v >= total) break;
        int s, x, y, z;
        digits(v, ns, gr.nx, gr.ny, s, x, y, z);
        double lx = 0.0, ly = 0.0;
        for (int k = 0; k < nb; k++) {
            const int e = st.entry[s * nb + k];
            const int xx = x + (e & 3) - 1, yy = y + ((e >> 2) & 3) - 1, zz = z + ((e >> 4) & 3) - 1;
            if (xx < 0 || xx >= gr.nx || yy < 0 || yy >= gr.ny || zz < 0 || zz >= gr.nz) continue;
            const long long o = (((long long)zz * gr.ny + yy) * gr.nx + xx) * ns + ((e >> 6) & 15);
            const double wk = gr.w[(e >> 10) & 3];
            lx += wk * double(f[2 * o]);
            ly += wk * double(f[2 * o + 1]);
        }
        const double px = double(f[2 * v]), py = double(f[2 * v + 1]);
        lx -= wsum * px;
        ly -= wsum * py;
        double V;
        if (vpot) {
            V = double(vpot[v]);
        } else {
            const double X = gr.origin[0] + gr.bs * (x * st.block_width + st.position[s][0]);
            const double Y = gr.origin[1] + gr.bs * (y * st.block_width + st.position[s][1]);
            const double Z = gr.origin[2] + gr.bs * (z * st.block_width + st.position[s][2]);
            V = 0.5 * (gr.trap[0] * X * X + gr.trap[1] * Y * Y + gr.trap[2] * Z * Z);
        }
        const double n2 = px * px + py * py;
        kahan(s0, c0, n2);
        kahan(s1, c1, -0.5 * (px * lx + py * ly));
        kahan(s2, c2, V * n2);
        kahan(s3, c3, 0.5 * gr.g * n2 * n2);
    }
    __shared__ double sm[4][kThreads];
    const int t = threadIdx.x;
    sm[0][t] = s0;
    sm[1][t] = s1;
    sm[2][t] = s2;
    sm[3][t] = s3;
    __syncthreads();
    for (int half = kThreads / 2; half > 0; half >>= 1) {
        if (t < half)
            for (int k = 0; k < 4; k++) sm[k][t] += sm[k][t + half];
        __syncthreads();
    }
    if (t < 6) rows[6ll * blockIdx.x + t] = t < 4 ? sm[t][0] : 0.0;
}

// The array's device address for the current device and context (first call
// in a context: look it up).
gpe_status scratch_for_current_device(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "gpe_observables_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(GPE_ERR_UNSUPPORTED, "gpe_observables_noalloc: device ordinal too high");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ScratchAddr &c = g_scratch_addr[dev];
    const unsigned long long id = current_context_id();
    if (id == 0 || c.ptr == nullptr || c.ctx_id != id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's primary context current if needed
        if (e != cudaSuccess) return cuda_fail(e, "gpe_observables_noalloc: cudaGetSymbolAddress");
        c.ptr = (double *)p;
        c.ctx_id = current_context_id();
    }
    *out = c.ptr;
    return GPE_OK;
}

}  // namespace
}  // namespace gpe

using namespace gpe;

static gpe_status gpe_observables_noalloc_impl(int32_t lattice, int32_t precision, const gpe_instance *inst,
                                               const void *field, const void *potential, void *stream,
                                               gpe_observables *out)
{
    if (!inst || !field || !out) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_observables_noalloc: null argument");
    if (lattice != GPE_LATTICE_TETRA12 && lattice != GPE_LATTICE_BCC2)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_observables_noalloc: unknown lattice");
    if (precision != GPE_FP64 && precision != GPE_FP32)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_observables_noalloc: unknown precision");
    if (inst->nx < 1 || inst->ny < 1 || inst->nz < 1 || !(inst->block_scale > 0.0))
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_observables_noalloc: bad grid");
    if (!g_stencils.ok) return fail(GPE_ERR_INTERNAL, "gpe_observables_noalloc: lattice tables unavailable");
    const NoallocStencil &st = g_stencils.s[lattice];
    const long long total = (long long)inst->nx * inst->ny * inst->nz * st.slots;
    if (total > (long long)kRows * kPerRow)
        return fail(GPE_ERR_TOO_LARGE, "gpe_observables_noalloc: more values than GPE_NOALLOC_MAX_ROWS * "
                                       "GPE_NOALLOC_VALUES_PER_ROW (16,777,216)");
    double *scratch = nullptr;
    gpe_status s = scratch_for_current_device(&scratch);
    if (s != GPE_OK) return s;
    NoallocGrid gr;
    gr.nx = inst->nx;
    gr.ny = inst->ny;
    gr.nz = inst->nz;
    const double s2 = inst->block_scale * inst->block_scale;
    gr.w[0] = st.cls_weight[0] / s2;
    gr.w[1] = st.cls_weight[1] / s2;
    gr.g = inst->g;
    gr.bs = inst->block_scale;
    for (int c = 0; c < 3; c++) {
        gr.origin[c] = inst->origin[c];
        gr.trap[c] = inst->trap[c];
    }
    cudaStream_t cs = (cudaStream_t)stream;
    const int ctas = int((total + kPerRow - 1) / kPerRow);
    if (precision == GPE_FP64)
        noalloc_observables_kernel<double><<<ctas, kThreads, 0, cs>>>(st, gr, (const double *)field,
                                                                      (const double *)potential, total);
    else
        noalloc_observables_kernel<float><<<ctas, kThreads, 0, cs>>>(st, gr, (const float *)field,
                                                                     (const float *)potential, total);
    GPE_CUDA_TRY(cudaGetLastError());
    GPE_CUDA_TRY(launch_reduce_partials(scratch, ctas, 6, scratch + 6ll * kRows, cs));
    double sums[6];
    GPE_CUDA_TRY(cudaMemcpyAsync(sums, scratch + 6ll * kRows, sizeof(sums), cudaMemcpyDeviceToHost, cs));
    GPE_CUDA_TRY(cudaStreamSynchronize(cs));
    const double vol = st.cell_volume * inst->block_scale * s2;
    out->norm = vol * sums[0];
    out->kinetic = vol * sums[1];
    out->potential = vol * sums[2];
    out->interaction = vol * sums[3];
    out->energy = out->kinetic + out->potential + out->interaction;
    out->mu = (out->kinetic + out->potential + 2.0 * out->interaction) / out->norm;
    out->finite = std::isfinite(out->norm) && std::isfinite(out->energy) && std::isfinite(out->mu);
    out->pad_ = 0;
    if (out->norm == 0.0)
        return fail(GPE_ERR_NOT_FINITE, "gpe_observables_noalloc: the field is zero everywhere (norm 0), so mu is "
                                        "undefined");
    if (!out->finite) return fail(GPE_ERR_NOT_FINITE, "gpe_observables_noalloc: NaN or Inf in the field");
    return GPE_OK;
}

extern "C" gpe_status gpe_observables_noalloc(int32_t lattice, int32_t precision, const gpe_instance *inst,
                                              const void *field, const void *potential, void *stream,
                                              gpe_observables *out)
{
    GPE_GUARD(gpe_observables_noalloc_impl(lattice, precision, inst, field, potential, stream, out));
}
