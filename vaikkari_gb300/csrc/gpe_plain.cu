// gpe_plain.cu - table-driven half-step for any lattice, one value per thread;
// FP64 observables; layout conversion.
//
// The plain step is the reference's update kernel (koodit/GrossPitaevskii/
// GPUGrossPitaevskii_BCC.cu:176-216) re-expressed for the padded slot-major
// layout: a warp covers 32 consecutive blocks along x of one slot, so every
// load of a neighbour slot is a coalesced 256/512-byte row segment (the
// reference's lanes are 192 bytes apart), and the neighbour table is read from
// constant memory with a warp-uniform index.

#include <cuda_runtime.h>

#include <cstring>

#include "gpe_internal.h"

namespace gpe {

// Packed neighbour entry: (dx+1) | (dy+1)<<2 | (dz+1)<<4 | slot<<6 | class<<10.
__constant__ int c_tab_tetra12[12 * 4];
__constant__ int c_tab_bcc2[2 * 14];

template <int LAT> struct Lat;
template <> struct Lat<GPE_LATTICE_TETRA12> {
    static constexpr int NS = 12, NB = 4, NC = 1, N0 = 4;
    __device__ static int entry(int k) { return c_tab_tetra12[k]; }
};
template <> struct Lat<GPE_LATTICE_BCC2> {
    static constexpr int NS = 2, NB = 14, NC = 2, N0 = 8;
    __device__ static int entry(int k) { return c_tab_bcc2[k]; }
};
// TETRA12 stepped in the face form: the faces and weights come from InstDev.
template <> struct Lat<kStepTetra12Faces> {
    static constexpr int NS = 12, NB = 4, NC = 1, N0 = 4;
    __device__ static int entry(int k) { return c_tab_tetra12[k]; }
};

// The face (Hodge) form of the reference's multi-GPU update
// (GPUGrossPitaevskii_BCC_multi.cu:329-397) for planes z0..z1-1 of one value:
//   sum = h_k (psi_k - psi) added over the four faces in summation order,
//   sum += (V dt + g dt |psi|^2) psi,   next += -i sum   (real time)
//                                       next = psi - sum (imaginary time).
// Each rounding is that kernel's as nvcc compiles it (fused multiply-add on by
// default): every h_k (psi_k - psi) is added with one fma, |psi|^2 is
// fma(x, x, y*y), V dt + g dt |psi|^2 one fma, and c psi is added with one fma.
template <typename T, int MODE, int POT>
__device__ __forceinline__ void face_values(const InstDev &d, const typename Cplx<T>::type *__restrict__ prev,
                                            typename Cplx<T>::type *__restrict__ next, const T *__restrict__ vpot,
                                            T sig, int s, int x, int y, int z0, int z1)
{
    using T2 = typename Cplx<T>::type;
    if constexpr (sizeof(T) == 8) {
        // FP64 is bound by the FP64 pipe: one value per thread (z1 = z0 + 1),
        // indices formed directly, fewest registers and most warps in flight.
        for (int z = z0; z < z1; z++) {
            const long long self = field_index(d, s, x, y, z);
            T2 p = prev[self];
            if (MODE == 1) p = c_scale<T>(sig, p);
            T sx = T(0), sy = T(0);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int e = d.fe[4 * s + k];
                const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
                T2 v = prev[field_index(d, sl, x + dx, y + dy, z + dz)];
                if (MODE == 1) v = c_scale<T>(sig, v);
                const T h = d.hf[4 * s + k];
                sx = d_fma(h, d_sub(v.x, p.x), sx);
                sy = d_fma(h, d_sub(v.y, p.y), sy);
            }
            T vdt;
            if (POT == GPE_POTENTIAL_ARRAY) vdt = vpot[self - d.base + d.vbase];
            else vdt = trap_vdt<T>(vpot, d, s, x, y, z);
            const T c = d_fma(T(d.gdt), d_fma(p.x, p.x, d_mul(p.y, p.y)), vdt);
            sx = d_fma(c, p.x, sx);
            sy = d_fma(c, p.y, sy);
            T2 n;
            if (MODE == 0) n = next[self];
            next[self] = integrate<T, MODE>(n, p, sx, sy);
        }
        return;
    }
    const long long base0 = field_index(d, s, x, y, 0);
    long long off[4];
    T h[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int e = d.fe[4 * s + k];
        const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
        off[k] = field_index(d, sl, x + dx, y + dy, dz) - base0;
        if constexpr (sizeof(T) == 8) h[k] = d.hf[4 * s + k];
        else h[k] = d.hf32[4 * s + k];
    }
    const T gdt = T(d.gdt);
    const long long voff = d.vbase - d.base;
    for (int z = z0; z < z1; z++) {
        const long long self = base0 + (long long)z * d.zstride;
        T2 p = prev[self];
        if (MODE == 1) p = c_scale<T>(sig, p);
        T sx = T(0), sy = T(0);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            T2 v = prev[self + off[k]];
            if (MODE == 1) v = c_scale<T>(sig, v);
            sx = d_fma(h[k], d_sub(v.x, p.x), sx);
            sy = d_fma(h[k], d_sub(v.y, p.y), sy);
        }
        T vdt;
        if (POT == GPE_POTENTIAL_ARRAY) vdt = vpot[self + voff];
        else vdt = trap_vdt<T>(vpot, d, s, x, y, z);
        const T c = d_fma(gdt, d_fma(p.x, p.x, d_mul(p.y, p.y)), vdt);
        sx = d_fma(c, p.x, sx);
        sy = d_fma(c, p.y, sy);
        T2 n;
        if (MODE == 0) n = next[self];
        next[self] = integrate<T, MODE>(n, p, sx, sy);
    }
}

cudaError_t set_plain_table(const gpe_lattice_info &info)
{
    int packed[12 * 14];
    const int nb = info.neighbours;
    for (int s = 0; s < info.slots; s++)
        for (int k = 0; k < nb; k++) {
            const int *e = info.entry[s][k];
            packed[s * nb + k] = (e[0] + 1) | ((e[1] + 1) << 2) | ((e[2] + 1) << 4) | (e[3] << 6) | (e[4] << 10);
        }
    if (info.lattice == GPE_LATTICE_TETRA12)
        return cudaMemcpyToSymbol(c_tab_tetra12, packed, sizeof(int) * 12 * 4);
    return cudaMemcpyToSymbol(c_tab_bcc2, packed, sizeof(int) * 2 * 14);
}

// vpot: the trap tables (POT == TRAP), or L0 + V*dt per value (POT == ARRAY).
// Thread (x, y) of a CTA handles value `slot` of block column (x, y) for the
// planes z0 .. z0+zc-1: the neighbours' offsets from the value are the same on
// every plane, so they are formed once and each plane only advances the index
// by one z-stride (the per-value arithmetic does not depend on this).
// (bx, bz): the CTA's block of the instance's grid (256 threads, bz = plane
// chunk * slots + slot).  The values of a slot's plane are numbered x fastest
// and CTA bx takes values 256 bx .. 256 bx + 255 of it, so that every warp but
// a plane's last is full.  (With 32 x 8 tiles, a plane whose nx is not a
// multiple of 32 left lanes idle in every warp of its last tile column - 87 of
// 96 lanes busy for nx = 87 - and those lanes still took issue slots and, in
// FP64, the FP64 pipe that bounds the path.)
template <typename T, int LAT, int MODE, int POT>
__device__ __forceinline__ void plain_step_body(const InstDev *__restrict__ insts, int ii,
                                                const typename Cplx<T>::type *__restrict__ prev,
                                                typename Cplx<T>::type *__restrict__ next,
                                                const T *__restrict__ vpot, const ImagScalars *__restrict__ imag, int zc,
                                                int bx, int bz)
{
    using T2 = typename Cplx<T>::type;
    using L = Lat<LAT>;
    const InstDev &d = insts[ii];
    const int l = bx * 256 + threadIdx.y * 32 + threadIdx.x;
    const int y = l / d.nx;
    const int x = l - y * d.nx;
    const int s = bz % L::NS;
    const int z0 = (bz / L::NS) * zc;
    if (x >= d.nx || y >= d.ny) return;
    const T sig = (MODE == 1) ? T(imag[ii].sigma) : T(1);
    if constexpr (LAT == kStepTetra12Faces) {
        face_values<T, MODE, POT>(d, prev, next, vpot, sig, s, x, y, z0, min(z0 + zc, d.nz));
        return;
    }
    if constexpr (sizeof(T) == 8) {
        // FP64 is bound by the FP64 pipe: one value per thread (zc == 1), indices
        // formed directly, fewest registers and most values in flight.
        const int z = z0;
        T2 S[L::NC];
#pragma unroll
        for (int k = 0; k < L::NB; k++) {
            const int e = L::entry(s * L::NB + k);
            const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
            T2 v = prev[field_index(d, sl, x + dx, y + dy, z + dz)];
            if (MODE == 1) v = c_scale<T>(sig, v);
            const int c = (k < L::N0) ? 0 : 1;
            if (k == 0 || k == L::N0) S[c] = v;
            else S[c] = c_add<T>(S[c], v);
        }
        const long long self = field_index(d, s, x, y, z);
        T2 p = prev[self];
        if (MODE == 1) p = c_scale<T>(sig, p);
        T vdt;
        if (POT == GPE_POTENTIAL_ARRAY) vdt = vpot[self - d.base + d.vbase];
        else vdt = trap_vdt<T>(vpot, d, s, x, y, z);
        T Lw[L::NC];
        Lw[0] = T(d.Lc[0]);
        if (L::NC > 1) Lw[L::NC - 1] = T(d.Lc[1]);
        T hx, hy, nrm;
        hpsi<T, L::NC, POT == GPE_POTENTIAL_ARRAY>(p, S, Lw, T(d.L0), vdt, T(d.gdt), hx, hy, nrm);
        T2 n;
        if (MODE == 0) n = next[self];
        next[self] = integrate<T, MODE>(n, p, hx, hy);
        return;
    }
    const int z1 = min(z0 + zc, d.nz);
    const long long base0 = field_index(d, s, x, y, 0);
    long long off[L::NB];
#pragma unroll
    for (int k = 0; k < L::NB; k++) {
        const int e = L::entry(s * L::NB + k);
        const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
        off[k] = field_index(d, sl, x + dx, y + dy, dz) - base0;
    }
    T Lw[L::NC];
    Lw[0] = T(d.Lc[0]);
    if (L::NC > 1) Lw[L::NC - 1] = T(d.Lc[1]);
    const T L0 = T(d.L0), gdt = T(d.gdt);
    const long long voff = d.vbase - d.base;
    for (int z = z0; z < z1; z++) {
        const long long self = base0 + (long long)z * d.zstride;
        T2 S[L::NC];
#pragma unroll
        for (int k = 0; k < L::NB; k++) {
            T2 v = prev[self + off[k]];
            if (MODE == 1) v = c_scale<T>(sig, v);
            const int c = (k < L::N0) ? 0 : 1;
            if (k == 0 || k == L::N0) S[c] = v;
            else S[c] = c_add<T>(S[c], v);
        }
        T2 p = prev[self];
        if (MODE == 1) p = c_scale<T>(sig, p);
        T vdt;
        if (POT == GPE_POTENTIAL_ARRAY) vdt = vpot[self + voff];
        else vdt = trap_vdt<T>(vpot, d, s, x, y, z);
        T hx, hy, nrm;
        hpsi<T, L::NC, POT == GPE_POTENTIAL_ARRAY>(p, S, Lw, L0, vdt, gdt, hx, hy, nrm);
        T2 n;
        if (MODE == 0) n = next[self];
        next[self] = integrate<T, MODE>(n, p, hx, hy);
    }
}

template <typename T, int LAT, int MODE, int POT>
__global__ void __launch_bounds__(256) plain_step_kernel(const InstDev *__restrict__ insts, int ii,
                                                         const typename Cplx<T>::type *__restrict__ prev,
                                                         typename Cplx<T>::type *__restrict__ next,
                                                         const T *__restrict__ vpot, const ImagScalars *__restrict__ imag,
                                                         int zc)
{
    plain_step_body<T, LAT, MODE, POT>(insts, ii, prev, next, vpot, imag, zc, blockIdx.x, blockIdx.z);
}

// CTAs of the plain kernel per slot plane: 256 consecutive values each.
__host__ __device__ inline int plain_plane_ctas(int nx, int ny) { return int(((long long)nx * ny + 255) / 256); }

int plain_blocks_per_plane(int nx, int ny) { return plain_plane_ctas(nx, ny); }

// Every instance of a batch in one launch: CTA b is block b - blk_begin[i] of
// instance i = blk_inst[b], numbered along the plane first, then z chunk and slot, as
// in that instance's own launch (same values per thread, same results).
template <typename T, int LAT, int MODE, int POT>
__global__ void __launch_bounds__(256) plain_step_batch_kernel(const InstDev *__restrict__ insts,
                                                               const int *__restrict__ blk_inst,
                                                               const int *__restrict__ blk_begin,
                                                               const int *__restrict__ zcs,
                                                               const typename Cplx<T>::type *__restrict__ prev,
                                                               typename Cplx<T>::type *__restrict__ next,
                                                               const T *__restrict__ vpot,
                                                               const ImagScalars *__restrict__ imag)
{
    const int i = blk_inst[blockIdx.x];
    const int local = blockIdx.x - blk_begin[i];
    const InstDev &d = insts[i];
    const int gx = plain_plane_ctas(d.nx, d.ny);
    const int rest = local / gx;
    plain_step_body<T, LAT, MODE, POT>(insts, i, prev, next, vpot, imag, zcs[i], local - rest * gx, rest);
}

// Planes per thread.  FP32 is issue-bound, so fewer index computations per value
// pay, the more so the larger the grid; FP64 is FP64-bound and wants many
// independent values in flight.  Measured with TETRA12 (value-updates/s):
//   32^3  (393 K values): FP32 2.4e10 / 3.2e10 / 3.2e10 for 1 / 2 / 4 planes
//   48^3  (1.3 M):        FP32 3.4e10 / 5.2e10 / 5.4e10 for 1 / 2 / 4
//   96^3  (10.6 M):       FP32 4.2e10 / 7.3e10 / 8.1e10 / 8.4e10 for 1 / 2 / 4 / 8
//   87x87x302 (27.4 M):   FP32 8.6e10 / 8.8e10 for 8 / 16; FP64 1.649e10 for 1-2, 1.62e10 for 16
// FP64 takes one value per thread in its own code path (32 registers, as many
// values in flight as possible); on 32^3 that path gives 1.22e10 against
// 1.14e10 for two planes per thread in the marching path.
static int plain_zchunk(long long values, bool fp64)
{
    if (fp64) return 1;
    if (values < (1ll << 20)) return 2;
    if (values < (4ll << 20)) return 4;
    if (values < (16ll << 20)) return 8;
    return 16;
}

template <typename T, int LAT>
static cudaError_t plain_dispatch_mode(const StepLaunch &l, cudaStream_t st)
{
    using T2 = typename Cplx<T>::type;
    const int zc = plain_zchunk((long long)l.nx * l.ny * l.nz * Lat<LAT>::NS, sizeof(T) == 8);
    dim3 block(32, 8, 1);
    dim3 grid(plain_plane_ctas(l.nx, l.ny), 1, ((l.nz + zc - 1) / zc) * Lat<LAT>::NS);
    const T2 *prev = (const T2 *)l.prev;
    T2 *next = (T2 *)l.next;
    const T *v = (const T *)(l.potential == GPE_POTENTIAL_ARRAY && LAT != kStepTetra12Faces ? l.vbase : l.vpot);
    if (l.mode == GPE_REAL_TIME) {
        if (l.potential == GPE_POTENTIAL_ARRAY)
            plain_step_kernel<T, LAT, 0, 0><<<grid, block, 0, st>>>(l.inst, l.inst_index, prev, next, v, l.imag, zc);
        else
            plain_step_kernel<T, LAT, 0, 1><<<grid, block, 0, st>>>(l.inst, l.inst_index, prev, next, v, l.imag, zc);
    } else {
        if (l.potential == GPE_POTENTIAL_ARRAY)
            plain_step_kernel<T, LAT, 1, 0><<<grid, block, 0, st>>>(l.inst, l.inst_index, prev, next, v, l.imag, zc);
        else
            plain_step_kernel<T, LAT, 1, 1><<<grid, block, 0, st>>>(l.inst, l.inst_index, prev, next, v, l.imag, zc);
    }
    return cudaGetLastError();
}

template <typename T>
__global__ void potential_base_kernel(const InstDev *__restrict__ insts, int ii, const T *__restrict__ vpot,
                                      T *__restrict__ vbase)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    const T L0 = T(d.L0);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int x, y, s, z;
        digits(v, d.nx, d.ny, d.slots, x, y, s, z);
        const long long o = field_index(d, s, x, y, z) - d.base + d.vbase;
        vbase[o] = d_add(L0, vpot[o]);  // the add hpsi would do every half-step
    }
}

cudaError_t launch_potential_base(int precision, const InstDev *inst, int ii, int nx, int ny, int nz, int slots,
                                  const void *vpot, void *vbase, cudaStream_t s)
{
    long long g = ((long long)nx * ny * nz * slots + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    if (precision == GPE_FP64)
        potential_base_kernel<double><<<int(g), 256, 0, s>>>(inst, ii, (const double *)vpot, (double *)vbase);
    else
        potential_base_kernel<float><<<int(g), 256, 0, s>>>(inst, ii, (const float *)vpot, (float *)vbase);
    return cudaGetLastError();
}

int plain_planes_per_thread(long long values, int precision) { return plain_zchunk(values, precision == GPE_FP64); }

template <typename T, int LAT>
static cudaError_t plain_batch_mode(const PlainBatchLaunch &l, cudaStream_t st)
{
    using T2 = typename Cplx<T>::type;
    const T2 *prev = (const T2 *)l.prev;
    T2 *next = (T2 *)l.next;
    const T *v = (const T *)(l.potential == GPE_POTENTIAL_ARRAY && LAT != kStepTetra12Faces ? l.vbase : l.vpot);
#define GPE_PB(MODE, POT) \
    plain_step_batch_kernel<T, LAT, MODE, POT><<<l.blocks, dim3(32, 8, 1), 0, st>>>(l.inst, l.blk_inst, l.blk_begin, \
                                                                                 l.zcs, prev, next, v, l.imag)
    const bool arr = l.potential == GPE_POTENTIAL_ARRAY;
    if (l.mode == GPE_REAL_TIME) { if (arr) GPE_PB(0, 0); else GPE_PB(0, 1); }
    else { if (arr) GPE_PB(1, 0); else GPE_PB(1, 1); }
#undef GPE_PB
    return cudaGetLastError();
}

cudaError_t launch_plain_step_batch(const PlainBatchLaunch &l, cudaStream_t s)
{
    if (l.precision == GPE_FP64) {
        if (l.lattice == GPE_LATTICE_TETRA12) return plain_batch_mode<double, GPE_LATTICE_TETRA12>(l, s);
        if (l.lattice == kStepTetra12Faces) return plain_batch_mode<double, kStepTetra12Faces>(l, s);
        if (l.lattice == GPE_LATTICE_BCC2) return plain_batch_mode<double, GPE_LATTICE_BCC2>(l, s);
        return cudaErrorInvalidValue;
    }
    if (l.lattice == GPE_LATTICE_TETRA12) return plain_batch_mode<float, GPE_LATTICE_TETRA12>(l, s);
    if (l.lattice == kStepTetra12Faces) return plain_batch_mode<float, kStepTetra12Faces>(l, s);
    if (l.lattice == GPE_LATTICE_BCC2) return plain_batch_mode<float, GPE_LATTICE_BCC2>(l, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_plain_step(const StepLaunch &l, cudaStream_t s)
{
    if (l.precision == GPE_FP64) {
        if (l.lattice == GPE_LATTICE_TETRA12) return plain_dispatch_mode<double, GPE_LATTICE_TETRA12>(l, s);
        if (l.lattice == kStepTetra12Faces) return plain_dispatch_mode<double, kStepTetra12Faces>(l, s);
        if (l.lattice == GPE_LATTICE_BCC2) return plain_dispatch_mode<double, GPE_LATTICE_BCC2>(l, s);
        return cudaErrorInvalidValue;
    }
    if (l.lattice == GPE_LATTICE_TETRA12) return plain_dispatch_mode<float, GPE_LATTICE_TETRA12>(l, s);
    if (l.lattice == kStepTetra12Faces) return plain_dispatch_mode<float, kStepTetra12Faces>(l, s);
    if (l.lattice == GPE_LATTICE_BCC2) return plain_dispatch_mode<float, GPE_LATTICE_BCC2>(l, s);
    return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Observables: per-value sums in FP64 with Kahan compensation per thread, a
// fixed-shape tree per CTA, one row of 6 partial sums per CTA.  Sums (without the
// volume factor): |psi|^2, Re(conj(psi)(-1/2 Lap psi)), V|psi|^2, g/2 |psi|^4,
// and two spares (0).

struct Kahan {
    double s = 0.0, c = 0.0;
    __device__ void add(double v)
    {
        const double y = v - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

template <int W>
__device__ void cta_tree_store(double (&v)[W], double *out)
{
    __shared__ double sm[W][256];
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < W; k++) sm[k][t] = v[k];
    __syncthreads();
    for (int half = 128; half > 0; half >>= 1) {
        if (t < half) {
#pragma unroll
            for (int k = 0; k < W; k++) sm[k][t] = sm[k][t] + sm[k][t + half];
        }
        __syncthreads();
    }
    if (t < W) out[t] = sm[t][0];
}

// Float pairs: a value hi + lo with |lo| <= ulp(hi)/2, carried by error-free
// transformations on the FP32 pipe (Knuth's two-sum; the two-product through
// fma).  Addition is the accurate form (both parts two-summed), whose error is
// about 2^-44 of the result even when the operands cancel; multiplication
// rounds once at about 2^-44.  On this GPU the FP32 pipe is 64 times the FP64
// pipe, so some twenty FP32 operations per double-precision step are cheaper
// than the FP64 instruction they replace.
struct FPair {
    float hi, lo;
};
__device__ __forceinline__ FPair fp_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FPair fp_fast_two_sum(float a, float b)  // |a| >= |b| or a == 0
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FPair fp_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ FPair fp_add(FPair x, FPair y)
{
    FPair s = fp_two_sum(x.hi, y.hi);
    const FPair t = fp_two_sum(x.lo, y.lo);
    s = fp_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fp_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ FPair fp_mul(FPair x, FPair y)
{
    const FPair p = fp_two_prod(x.hi, y.hi);
    return fp_fast_two_sum(p.hi, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo)));
}
__device__ __forceinline__ FPair fp_scale(FPair x, float k)  // k a power of two: exact
{
    return {__fmul_rn(x.hi, k), __fmul_rn(x.lo, k)};
}
__device__ __forceinline__ FPair fp_of(double v)
{
    const float hi = __double2float_rn(v);
    return {hi, __double2float_rn(__dsub_rn(v, double(hi)))};
}
__device__ __forceinline__ double fp_value(FPair x) { return __dadd_rn(double(x.hi), double(x.lo)); }

// The same pairs for the two components of a complex value at once: each
// packed f32x2 operation is the two scalar operations of its lanes, so a pair of
// float2 carries (re, im) through exactly the arithmetic of two FPairs.
struct FPair2 {
    float2 hi, lo;
};
__device__ __forceinline__ float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ FPair2 fp2_two_sum(float2 a, float2 b)
{
    const float2 s = f2_add(a, b);
    const float2 bb = f2_sub(s, a);
    return {s, f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb))};
}
__device__ __forceinline__ FPair2 fp2_fast_two_sum(float2 a, float2 b)
{
    const float2 s = f2_add(a, b);
    return {s, f2_sub(b, f2_sub(s, a))};
}
__device__ __forceinline__ FPair2 fp2_two_prod(float2 a, float2 b)
{
    const float2 p = f2_mul(a, b);
    return {p, f2_fma(a, b, f2_neg(p))};
}
__device__ __forceinline__ FPair2 fp2_add(FPair2 x, FPair2 y)
{
    FPair2 s = fp2_two_sum(x.hi, y.hi);
    const FPair2 t = fp2_two_sum(x.lo, y.lo);
    s = fp2_fast_two_sum(s.hi, f2_add(s.lo, t.hi));
    return fp2_fast_two_sum(s.hi, f2_add(s.lo, t.lo));
}
__device__ __forceinline__ FPair2 fp2_mul(FPair2 x, FPair2 y)
{
    const FPair2 p = fp2_two_prod(x.hi, y.hi);
    return fp2_fast_two_sum(p.hi, f2_fma(x.hi, y.lo, f2_fma(x.lo, y.hi, p.lo)));
}

// The observables of FP32 values, all in float-pair arithmetic: per class c
// the neighbour sum S_c as an error-free pair, the bracket S_c - n_c psi (the
// Laplacian's cancellation, exact up to the pair's rounding), Lap psi =
// sum_c w_c (S_c - n_c psi), and the four terms, each added into a float-pair
// accumulator.  Agrees with FP64 evaluation to about 1e-13 relative.  The
// per-neighbour and per-class work runs on both components at once (FPair2).
template <int LAT, int POT>
__device__ __forceinline__ void observables_terms_f32(const InstDev &d, const float2 *__restrict__ f,
                                                      const float *__restrict__ vpot, int s, int x, int y, int z,
                                                      long long self, const long long *__restrict__ off,
                                                      const FPair (&w)[2], FPair rdt, FPair half_g, FPair2 (&acc)[2])
{
    using L = Lat<LAT>;
    const float2 pt = f[self];
    const float2 zero = make_float2(0.f, 0.f);
    float2 h[2] = {zero, zero}, l[2] = {zero, zero};
#pragma unroll
    for (int k = 0; k < L::NB; k++) {
        const float2 q = f[self + off[k]];
        const int c = (k < L::N0) ? 0 : 1;
        const FPair2 t = fp2_two_sum(h[c], q);
        h[c] = t.hi;
        l[c] = f2_add(l[c], t.lo);
    }
    FPair2 lap = {zero, zero};
#pragma unroll
    for (int c = 0; c < L::NC; c++) {
        const float n = float(c == 0 ? L::N0 : L::NB - L::N0);
        const FPair2 np = fp2_two_prod(make_float2(n, n), pt);
        const FPair2 b = fp2_add(fp2_two_sum(h[c], l[c]), {f2_neg(np.hi), f2_neg(np.lo)});
        lap = fp2_add(lap, fp2_mul({make_float2(w[c].hi, w[c].hi), make_float2(w[c].lo, w[c].lo)}, b));
    }
    float vdt;
    if (POT == GPE_POTENTIAL_ARRAY) vdt = vpot[self - d.base + d.vbase];
    else vdt = trap_vdt<float>(vpot, d, s, x, y, z);
    // The four terms, two at a time: lane pairs (re, im), then (norm, kinetic)
    // and (potential, interaction) - each lane the scalar pair arithmetic.
    const FPair2 sq = fp2_two_prod(pt, pt);                          // x^2, y^2
    const FPair n2 = fp_add({sq.hi.x, sq.lo.x}, {sq.hi.y, sq.lo.y});
    const FPair2 pl = fp2_mul({pt, zero}, lap);                      // x Lap_x, y Lap_y
    const FPair kin = fp_scale(fp_add({pl.hi.x, pl.lo.x}, {pl.hi.y, pl.lo.y}), -0.5f);
    acc[0] = fp2_add(acc[0], {make_float2(n2.hi, kin.hi), make_float2(n2.lo, kin.lo)});
    // (vdt * rdt, n2 * n2), then (that * n2, half_g * n2^2)
    const FPair2 m1 = fp2_mul({make_float2(vdt, n2.hi), make_float2(0.f, n2.lo)},
                              {make_float2(rdt.hi, n2.hi), make_float2(rdt.lo, n2.lo)});
    const FPair2 m2 = fp2_mul({make_float2(m1.hi.x, half_g.hi), make_float2(m1.lo.x, half_g.lo)},
                              {make_float2(n2.hi, m1.hi.y), make_float2(n2.lo, m1.lo.y)});
    acc[1] = fp2_add(acc[1], m2);
}

// One CTA's share of one instance's sums: values first, first + stride, ...;
// writes the CTA's row of 6 partial sums to `row`.
template <typename T, int LAT, int POT>
__device__ __forceinline__ void observables_body(const InstDev &d, const typename Cplx<T>::type *__restrict__ f,
                                                 const T *__restrict__ vpot, long long first, long long stride,
                                                 double *__restrict__ row)
{
    using T2 = typename Cplx<T>::type;
    using L = Lat<LAT>;
    const long long total = (long long)d.nx * d.ny * d.nz * L::NS;
    Kahan k0, k1, k2, k3;
    const double wsum = L::N0 * d.w[0] + (L::NB - L::N0) * d.w[1];
    const double rdt = 1.0 / d.dt;
    // neighbour k of a value in slot s sits nb_off[s * NB + k] places from it
    // (the CTA's instance; the lattice form's table)
    __shared__ long long nb_off[L::NS * L::NB];
    for (int i = threadIdx.x; i < L::NS * L::NB; i += blockDim.x) {
        const int e = L::entry(i), sl0 = i / L::NB;
        const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
        nb_off[i] = (long long)dz * d.zstride + (long long)(sl - sl0) * d.plane + (long long)dy * d.px + dx;
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4 && LAT != kStepTetra12Faces) {
        if (!(LAT == GPE_LATTICE_TETRA12 && d.face)) {
            const FPair w[2] = {fp_of(d.w[0]), fp_of(d.w[1])};
            const FPair rdt2 = fp_of(rdt), half_g = fp_of(0.5 * d.g);
            // (norm, kinetic) and (potential, interaction) float pairs
            FPair2 acc[2] = {{make_float2(0.f, 0.f), make_float2(0.f, 0.f)},
                             {make_float2(0.f, 0.f), make_float2(0.f, 0.f)}};
            for (long long v = first; v < total; v += stride) {
                int x, y, s, z;
                digits(v, d.nx, d.ny, L::NS, x, y, s, z);
                observables_terms_f32<LAT, POT>(d, (const float2 *)f, (const float *)vpot, s, x, y, z,
                                                field_index(d, s, x, y, z), nb_off + s * L::NB, w, rdt2, half_g,
                                                acc);
            }
            double out[6] = {fp_value({acc[0].hi.x, acc[0].lo.x}), fp_value({acc[0].hi.y, acc[0].lo.y}),
                             fp_value({acc[1].hi.x, acc[1].lo.x}), fp_value({acc[1].hi.y, acc[1].lo.y}), 0.0, 0.0};
            cta_tree_store<6>(out, row);
            return;
        }
    }
    for (long long v = first; v < total; v += stride) {
        int x, y, s, z;
        digits(v, d.nx, d.ny, L::NS, x, y, s, z);
        const long long self = field_index(d, s, x, y, z);
        const T2 pt = f[self];
        const double px = double(pt.x), py = double(pt.y);
        double lx, ly;
        if (LAT == GPE_LATTICE_TETRA12 && d.face) {
            // face form: Lap psi = sum_k (hodge_k / bs^2) (psi_k - psi)
            lx = 0.0;
            ly = 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int e = d.fe[4 * s + k];
                const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
                const T2 q = f[field_index(d, sl, x + dx, y + dy, z + dz)];
                lx += d.hw[4 * s + k] * (double(q.x) - px);
                ly += d.hw[4 * s + k] * (double(q.y) - py);
            }
        } else {
            double sx[2] = {0.0, 0.0}, sy[2] = {0.0, 0.0};
            if constexpr (sizeof(T) == 4) {
                // FP32 values: each class sum kept as an unevaluated float pair
                // (hi + lo, error-free two-sums, lo accumulated in FP32) and
                // converted once, so the FP64 pipe (slow on this GPU) sees a few
                // operations per value instead of a conversion and an add per
                // neighbour.  Agrees with FP64 summation to about 1e-14.
                float hx[2] = {0.f, 0.f}, lx_[2] = {0.f, 0.f}, hy[2] = {0.f, 0.f}, ly_[2] = {0.f, 0.f};
#pragma unroll
                for (int k = 0; k < L::NB; k++) {
                    const T2 q = f[self + nb_off[s * L::NB + k]];
                    const int c = (k < L::N0) ? 0 : 1;
                    float t = __fadd_rn(hx[c], q.x), bb = __fsub_rn(t, hx[c]);
                    lx_[c] = __fadd_rn(lx_[c], __fadd_rn(__fsub_rn(hx[c], __fsub_rn(t, bb)), __fsub_rn(q.x, bb)));
                    hx[c] = t;
                    t = __fadd_rn(hy[c], q.y);
                    bb = __fsub_rn(t, hy[c]);
                    ly_[c] = __fadd_rn(ly_[c], __fadd_rn(__fsub_rn(hy[c], __fsub_rn(t, bb)), __fsub_rn(q.y, bb)));
                    hy[c] = t;
                }
#pragma unroll
                for (int c = 0; c < L::NC; c++) {
                    sx[c] = double(hx[c]) + double(lx_[c]);
                    sy[c] = double(hy[c]) + double(ly_[c]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < L::NB; k++) {
                    const T2 q = f[self + nb_off[s * L::NB + k]];
                    const int c = (k < L::N0) ? 0 : 1;
                    sx[c] += double(q.x);
                    sy[c] += double(q.y);
                }
            }
            lx = d.w[0] * sx[0] + d.w[1] * sx[1] - wsum * px;
            ly = d.w[0] * sy[0] + d.w[1] * sy[1] - wsum * py;
        }
        double vdt;
        if (POT == GPE_POTENTIAL_ARRAY) vdt = double(vpot[self - d.base + d.vbase]);
        else vdt = double(trap_vdt<T>(vpot, d, s, x, y, z));
        const double n2 = px * px + py * py;
        k0.add(n2);
        k1.add(-0.5 * (px * lx + py * ly));
        k2.add((vdt * rdt) * n2);
        k3.add(0.5 * d.g * n2 * n2);
    }
    double acc[6] = {k0.s, k1.s, k2.s, k3.s, 0.0, 0.0};
    cta_tree_store<6>(acc, row);
}

template <typename T, int LAT, int POT>
__global__ void __launch_bounds__(256) observables_kernel(const InstDev *__restrict__ insts, int ii,
                                                          const typename Cplx<T>::type *__restrict__ f,
                                                          const T *__restrict__ vpot, double *__restrict__ partials)
{
    observables_body<T, LAT, POT>(insts[ii], f, vpot, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                                  (long long)gridDim.x * blockDim.x, partials + 6ll * blockIdx.x);
}

// Every instance in one launch: CTA b belongs to instance cta_inst[b] and is its
// (b - cta_begin[i])-th CTA of cta_begin[i+1] - cta_begin[i]
// (observables_batch_ctas), covering values first, first + stride, ... of the
// instance as in its own launch, with fewer, longer-lived CTAs.
template <typename T, int LAT, int POT>
__global__ void __launch_bounds__(256) observables_batch_kernel(const InstDev *__restrict__ insts,
                                                                const int *__restrict__ cta_inst,
                                                                const int *__restrict__ cta_begin,
                                                                const typename Cplx<T>::type *__restrict__ f,
                                                                const T *__restrict__ vpot,
                                                                double *__restrict__ partials)
{
    const int i = cta_inst[blockIdx.x];
    const int b = cta_begin[i], n = cta_begin[i + 1] - b;
    observables_body<T, LAT, POT>(insts[i], f, vpot, (long long)(blockIdx.x - b) * blockDim.x + threadIdx.x,
                                  (long long)n * blockDim.x, partials + 6ll * blockIdx.x);
}

cudaError_t launch_observables(const ObsLaunch &l, cudaStream_t s, int *ctas_used)
{
    const long long total = (long long)l.nx * l.ny * l.nz * l.slots;
    const int ctas = observables_ctas(total, l.max_ctas);
    *ctas_used = ctas;
#define GPE_OBS(T, LAT, POT) \
    observables_kernel<T, LAT, POT><<<ctas, 256, 0, s>>>(l.inst, l.inst_index, (const Cplx<T>::type *)l.field, (const T *)l.vpot, l.partials)
    const bool arr = l.potential == GPE_POTENTIAL_ARRAY;
    if (l.precision == GPE_FP64) {
        if (l.lattice == GPE_LATTICE_TETRA12) { if (arr) GPE_OBS(double, 0, 0); else GPE_OBS(double, 0, 1); }
        else { if (arr) GPE_OBS(double, 1, 0); else GPE_OBS(double, 1, 1); }
    } else {
        if (l.lattice == GPE_LATTICE_TETRA12) { if (arr) GPE_OBS(float, 0, 0); else GPE_OBS(float, 0, 1); }
        else { if (arr) GPE_OBS(float, 1, 0); else GPE_OBS(float, 1, 1); }
    }
#undef GPE_OBS
    return cudaGetLastError();
}

// One CTA: thread t folds rows t, t+256, ... with Kahan, then a fixed tree.
__global__ void __launch_bounds__(256) reduce_partials_kernel(const double *__restrict__ partials, int rows, int width,
                                                              double *__restrict__ out)
{
    double acc[6];
    for (int k = 0; k < 6; k++) {
        Kahan kk;
        if (k < width)
            for (int r = threadIdx.x; r < rows; r += 256) kk.add(partials[(long long)r * width + k]);
        acc[k] = kk.s;
    }
    cta_tree_store<6>(acc, out);
}

int observables_ctas(long long values, int max_ctas)
{
    long long want = (values + 255) / 256;
    int ctas = int(want < max_ctas ? want : max_ctas);
    return ctas < 1 ? 1 : ctas;
}

// In the batched launch the instances' CTAs run together, so each instance gets
// one CTA per 4096 values (16 per thread): a CTA then spends most of its life on
// values rather than on its closing tree of partial sums (one value per thread
// left the warps waiting at that tree's barriers for most of the launch).
int observables_batch_ctas(long long values, int max_ctas)
{
    long long want = (values + kObsValuesPerBatchCta - 1) / kObsValuesPerBatchCta;
    int ctas = int(want < max_ctas ? want : max_ctas);
    return ctas < 1 ? 1 : ctas;
}

cudaError_t launch_observables_batch(int lattice, int precision, int potential, const InstDev *inst,
                                     const int *cta_inst, const int *cta_begin, int total_ctas, const void *field,
                                     const void *vpot, double *partials, cudaStream_t s)
{
#define GPE_OBSB(T, LAT, POT)                                                                                     \
    observables_batch_kernel<T, LAT, POT><<<total_ctas, 256, 0, s>>>(inst, cta_inst, cta_begin,                 \
                                                                      (const Cplx<T>::type *)field, (const T *)vpot, \
                                                                      partials)
    const bool arr = potential == GPE_POTENTIAL_ARRAY;
    if (precision == GPE_FP64) {
        if (lattice == GPE_LATTICE_TETRA12) { if (arr) GPE_OBSB(double, 0, 0); else GPE_OBSB(double, 0, 1); }
        else { if (arr) GPE_OBSB(double, 1, 0); else GPE_OBSB(double, 1, 1); }
    } else {
        if (lattice == GPE_LATTICE_TETRA12) { if (arr) GPE_OBSB(float, 0, 0); else GPE_OBSB(float, 0, 1); }
        else { if (arr) GPE_OBSB(float, 1, 0); else GPE_OBSB(float, 1, 1); }
    }
#undef GPE_OBSB
    return cudaGetLastError();
}

// One CTA per instance: instance i's rows cta_begin[i] .. cta_begin[i+1]-1, folded
// exactly as reduce_partials_kernel folds one instance's rows.
__global__ void __launch_bounds__(256) reduce_partials_batch_kernel(const double *__restrict__ partials,
                                                                    const int *__restrict__ cta_begin,
                                                                    double *__restrict__ out)
{
    const int i = blockIdx.x;
    const int b = cta_begin[i], rows = cta_begin[i + 1] - b;
    double acc[6];
    for (int k = 0; k < 6; k++) {
        Kahan kk;
        for (int r = threadIdx.x; r < rows; r += 256) kk.add(partials[(long long)(b + r) * 6 + k]);
        acc[k] = kk.s;
    }
    cta_tree_store<6>(acc, out + 6ll * i);
}

cudaError_t launch_reduce_partials_batch(const double *partials, const int *cta_begin, int instances, double *out,
                                         cudaStream_t s)
{
    reduce_partials_batch_kernel<<<instances, 256, 0, s>>>(partials, cta_begin, out);
    return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const double *partials, int ctas, int width, double *out, cudaStream_t s)
{
    reduce_partials_kernel<<<1, 256, 0, s>>>(partials, ctas, width, out);
    return cudaGetLastError();
}

__global__ void imag_finalize_plain_kernel(const double *__restrict__ sums, const InstDev *__restrict__ insts, int ii,
                                           ImagScalars *__restrict__ imag, double tol)
{
    const InstDev &d = insts[ii];
    ImagScalars &st = imag[ii];
    const double n = d.vol * sums[0];
    const double kin = d.vol * sums[1], pot = d.vol * sums[2], inter = d.vol * sums[3];
    // Observables of the normalised field sigma*psi, sigma^2 = 1/n.
    const double mu = (kin + pot) / n + 2.0 * inter / (n * n);
    st.sigma = 1.0 / sqrt(n);
    st.norm_in = n;
    st.energy = (kin + pot) / n + inter / (n * n);
    st.mu_prev = st.mu;
    st.mu = mu;
    st.dmu = (st.steps > 0) ? fabs(mu - st.mu_prev) : INFINITY;
    if (st.steps > 0 && st.conv_step < 0 && st.dmu < tol) st.conv_step = st.steps;
    st.steps += 1;
}

cudaError_t launch_imag_finalize_plain(const double *sums, const InstDev *inst, int inst_index, ImagScalars *imag,
                                       double tol, const long long *, cudaStream_t s)
{
    imag_finalize_plain_kernel<<<1, 1, 0, s>>>(sums, inst, inst_index, imag, tol);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Layout conversion.  Host order: (((z*ny)+y)*nx+x)*slots+s.

template <typename T, bool CPLX>
__global__ void pack_kernel(const InstDev *__restrict__ insts, int ii, const T *__restrict__ src, T *__restrict__ dst,
                            double scale)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int s, x, y, z;
        digits(v, d.slots, d.nx, d.ny, s, x, y, z);
        if (CPLX) {
            const long long o = field_index(d, s, x, y, z);
            ((typename Cplx<T>::type *)dst)[o] = ((const typename Cplx<T>::type *)src)[v];
        } else {
            const long long o = field_index(d, s, x, y, z) - d.base + d.vbase;
            dst[o] = T(double(src[v]) * scale);
        }
    }
}

template <typename T>
__global__ void unpack_kernel(const InstDev *__restrict__ insts, int ii, const T *__restrict__ src, T *__restrict__ dst,
                              const ImagScalars *__restrict__ imag)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    const T sig = imag ? T(imag[ii].sigma) : T(1);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int s, x, y, z;
        digits(v, d.slots, d.nx, d.ny, s, x, y, z);
        const long long o = field_index(d, s, x, y, z);
        typename Cplx<T>::type q = ((const typename Cplx<T>::type *)src)[o];
        if (imag) {
            q.x = d_mul(sig, q.x);
            q.y = d_mul(sig, q.y);
        }
        ((typename Cplx<T>::type *)dst)[v] = q;
    }
}

template <typename T>
__global__ void scale_field_kernel(const InstDev *__restrict__ insts, int ii, T *__restrict__ f,
                                   const ImagScalars *__restrict__ imag)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    const T sig = T(imag[ii].sigma);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int x, y, s, z;
        digits(v, d.nx, d.ny, d.slots, x, y, s, z);
        const long long o = field_index(d, s, x, y, z);
        f[2 * o] = d_mul(sig, f[2 * o]);
        f[2 * o + 1] = d_mul(sig, f[2 * o + 1]);
    }
}

// Host value -> FP32 value hi and the part below it, r = float(x - hi) (x - hi is
// exact in double).  A float host value is its own hi; its r is hi - hi (zero,
// or NaN for Inf/NaN as in the double form) with no FP64 arithmetic, which runs
// at a small fraction of the FP32 rate on this GPU.
__device__ __forceinline__ void comp_split(double x, float &hi, float &r)
{
    hi = __double2float_rn(x);
    r = __double2float_rn(x - double(hi));
}
__device__ __forceinline__ void comp_split(float x, float &hi, float &r)
{
    hi = x;
    r = __fsub_rn(x, x);
}
// hi + lo rounded once to the host type.  For float the exact sum (hi and lo
// span at most 33 significant bits, so double holds it) rounded to float is the
// correctly rounded float sum, which __fadd_rn gives directly.
template <typename H> __device__ __forceinline__ H comp_join(float hi, float lo);
template <> __device__ __forceinline__ double comp_join<double>(float hi, float lo)
{
    return double(hi) + double(lo);
}
template <> __device__ __forceinline__ float comp_join<float>(float hi, float lo) { return __fadd_rn(hi, lo); }

// GPE_FP32C transfers.  Upload: a double x becomes hi = float(x) and the int8
// residual of float(x - hi) (x - hi is exact in double) in units of ulp(hi)/256;
// download: double(hi) + double(residual).  lo holds both components in one
// 16-bit word, re in the low byte.
template <typename H>  // host element: double, or float (the residual starts at zero)
__global__ void pack_split_kernel(const InstDev *__restrict__ insts, int ii, const H *__restrict__ src,
                                  float *__restrict__ hi, uint16_t *__restrict__ lo)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int s, x, y, z;
        digits(v, d.slots, d.nx, d.ny, s, x, y, z);
        const long long o = field_index(d, s, x, y, z);
        const typename Cplx<H>::type hv = ((const typename Cplx<H>::type *)src)[v];
        float ha, hb, ra, rb;
        comp_split(hv.x, ha, ra);
        comp_split(hv.y, hb, rb);
        ((float2 *)hi)[o] = make_float2(ha, hb);
        // residual = the part of the value below FP32, in units of ulp(hi) / 256
        lo[o - kLoShift] = uint16_t(comp_encode(ra, ha) | (comp_encode(rb, hb) << 8));
    }
}

template <typename H>  // host element: double, or float (value + residual rounded once)
__global__ void unpack_join_kernel(const InstDev *__restrict__ insts, int ii, const float *__restrict__ hi,
                                   const uint16_t *__restrict__ lo, H *__restrict__ dst)
{
    const InstDev &d = insts[ii];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        int s, x, y, z;
        digits(v, d.slots, d.nx, d.ny, s, x, y, z);
        const long long o = field_index(d, s, x, y, z);
        const uint32_t w = lo[o - kLoShift];
        const float2 hv = ((const float2 *)hi)[o];
        const float ha = hv.x, hb = hv.y;
        const float2 lf = make_float2(comp_decode(w, ha), comp_decode(w >> 8, hb));
        typename Cplx<H>::type out;
        out.x = comp_join<H>(ha, lf.x);
        out.y = comp_join<H>(hb, lf.y);
        ((typename Cplx<H>::type *)dst)[v] = out;
    }
}

static int grid_for(long long total)
{
    long long g = (total + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    return int(g < 1 ? 1 : g);
}

cudaError_t launch_pack(int precision, const InstDev *inst, int ii, int nx, int ny, int nz, int slots,
                        const void *host_order, void *field, int is_complex, double scale, cudaStream_t s)
{
    const int g = grid_for((long long)nx * ny * nz * slots);
    if (precision == GPE_FP64) {
        if (is_complex) pack_kernel<double, true><<<g, 256, 0, s>>>(inst, ii, (const double *)host_order, (double *)field, scale);
        else pack_kernel<double, false><<<g, 256, 0, s>>>(inst, ii, (const double *)host_order, (double *)field, scale);
    } else {
        if (is_complex) pack_kernel<float, true><<<g, 256, 0, s>>>(inst, ii, (const float *)host_order, (float *)field, scale);
        else pack_kernel<float, false><<<g, 256, 0, s>>>(inst, ii, (const float *)host_order, (float *)field, scale);
    }
    return cudaGetLastError();
}

cudaError_t launch_unpack(int precision, const InstDev *inst, int ii, int nx, int ny, int nz, int slots,
                          const void *field, void *host_order, const ImagScalars *imag, cudaStream_t s)
{
    const int g = grid_for((long long)nx * ny * nz * slots);
    if (precision == GPE_FP64)
        unpack_kernel<double><<<g, 256, 0, s>>>(inst, ii, (const double *)field, (double *)host_order, imag);
    else
        unpack_kernel<float><<<g, 256, 0, s>>>(inst, ii, (const float *)field, (float *)host_order, imag);
    return cudaGetLastError();
}

cudaError_t launch_pack_split(const InstDev *inst, int ii, int nx, int ny, int nz, int slots, const void *host_order,
                              void *field, void *lo, bool host_fp32, cudaStream_t s)
{
    const int g = grid_for((long long)nx * ny * nz * slots);
    if (host_fp32)
        pack_split_kernel<float><<<g, 256, 0, s>>>(inst, ii, (const float *)host_order, (float *)field, (uint16_t *)lo);
    else
        pack_split_kernel<double><<<g, 256, 0, s>>>(inst, ii, (const double *)host_order, (float *)field,
                                                    (uint16_t *)lo);
    return cudaGetLastError();
}

cudaError_t launch_unpack_join(const InstDev *inst, int ii, int nx, int ny, int nz, int slots, const void *field,
                               const void *lo, void *host_order, bool host_fp32, cudaStream_t s)
{
    const int g = grid_for((long long)nx * ny * nz * slots);
    if (host_fp32)
        unpack_join_kernel<float><<<g, 256, 0, s>>>(inst, ii, (const float *)field, (const uint16_t *)lo,
                                                    (float *)host_order);
    else
        unpack_join_kernel<double><<<g, 256, 0, s>>>(inst, ii, (const float *)field, (const uint16_t *)lo,
                                                     (double *)host_order);
    return cudaGetLastError();
}

// ---- Batched transfers: every instance's fields in one launch ---------------
// Segment k (one field of one instance) owns CTAs segs[k].cta0 .. segs[k+1].cta0
// - 1 and converts between its host buffer, which the kernel reads or writes in
// place over the host link, and the padded device layout, with the arithmetic
// of pack_kernel / unpack_kernel (plain storage) or pack_split_kernel /
// unpack_join_kernel (GPE_FP32C).  One launch instead of one per field keeps the
// host link busy from the first segment to the last.
struct XferFields {
    void *field[2];
    uint16_t *lo[2];
};

template <typename T, typename H, bool COMP, bool UP>
__global__ void __launch_bounds__(256) xfer_batch_kernel(const InstDev *__restrict__ insts,
                                                         const XferSeg *__restrict__ segs, int nseg, XferFields fl)
{
    int a = 0, b = nseg - 1;  // the last segment whose first CTA is <= this one
    while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (segs[m].cta0 <= int(blockIdx.x)) a = m;
        else b = m - 1;
    }
    const XferSeg g = segs[a];
    const int ctas = segs[a + 1].cta0 - g.cta0;
    const InstDev &d = insts[g.inst];
    const long long total = (long long)d.nx * d.ny * d.nz * d.slots;
    using T2 = typename Cplx<T>::type;
    using H2 = typename Cplx<H>::type;
    T2 *__restrict__ field = (T2 *)fl.field[g.field];
    uint16_t *__restrict__ lo = fl.lo[g.field];
    // Each thread's values v0, v0 + step, ...: the host reads of an upload are
    // issued together (kXferValuesPerCta / 256 of them in flight per thread),
    // then converted and stored.
    constexpr int K = kXferValuesPerCta / 256;
    const long long step = (long long)ctas * blockDim.x;
    const long long v0 = (long long)(blockIdx.x - g.cta0) * blockDim.x + threadIdx.x;
    H2 hin[K];
    if constexpr (UP) {
#pragma unroll
        for (int k = 0; k < K; k++)
            if (v0 + k * step < total) hin[k] = ((const H2 *)g.host)[v0 + k * step];
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        const long long v = v0 + k * step;
        if (v >= total) break;
        int s, x, y, z;
        digits(v, d.slots, d.nx, d.ny, s, x, y, z);
        const long long o = field_index(d, s, x, y, z);
        if constexpr (UP && COMP) {
            const H2 hv = hin[k];
            float ha, hb, ra, rb;
            comp_split(hv.x, ha, ra);
            comp_split(hv.y, hb, rb);
            field[o] = make_float2(ha, hb);
            lo[o - kLoShift] = uint16_t(comp_encode(ra, ha) | (comp_encode(rb, hb) << 8));
        } else if constexpr (UP) {
            field[o] = hin[k];
        } else if constexpr (COMP) {
            const uint32_t w = lo[o - kLoShift];
            const float2 hv = field[o];
            H2 out;
            out.x = comp_join<H>(hv.x, comp_decode(w, hv.x));
            out.y = comp_join<H>(hv.y, comp_decode(w >> 8, hv.y));
            ((H2 *)g.host)[v] = out;
        } else {
            ((T2 *)g.host)[v] = field[o];
        }
    }
}

cudaError_t launch_xfer_batch(int precision, bool comp, bool host_fp32, bool up, const InstDev *inst,
                              const XferSeg *segs, int nseg, int ctas, void *field0, void *field1, void *lo0, void *lo1,
                              cudaStream_t s)
{
    const XferFields fl = {{field0, field1}, {(uint16_t *)lo0, (uint16_t *)lo1}};
#define GPE_XB(T, H, C, U) xfer_batch_kernel<T, H, C, U><<<ctas, 256, 0, s>>>(inst, segs, nseg, fl)
    if (comp) {
        if (host_fp32) { if (up) GPE_XB(float, float, true, true); else GPE_XB(float, float, true, false); }
        else { if (up) GPE_XB(float, double, true, true); else GPE_XB(float, double, true, false); }
    } else if (precision == GPE_FP64) {
        if (up) GPE_XB(double, double, false, true); else GPE_XB(double, double, false, false);
    } else {
        if (up) GPE_XB(float, float, false, true); else GPE_XB(float, float, false, false);
    }
#undef GPE_XB
    return cudaGetLastError();
}

cudaError_t launch_scale_field(int precision, const InstDev *inst, int ii, int nx, int ny, int nz, int slots,
                               void *field, const ImagScalars *imag, cudaStream_t s)
{
    const int g = grid_for((long long)nx * ny * nz * slots);
    if (precision == GPE_FP64) scale_field_kernel<double><<<g, 256, 0, s>>>(inst, ii, (double *)field, imag);
    else scale_field_kernel<float><<<g, 256, 0, s>>>(inst, ii, (float *)field, imag);
    return cudaGetLastError();
}

__global__ void imag_init_kernel(const double *__restrict__ sums, const InstDev *__restrict__ insts, int ii,
                                 ImagScalars *__restrict__ imag)
{
    const double n = insts[ii].vol * sums[0];
    imag[ii].sigma = 1.0 / sqrt(n);
    imag[ii].norm_in = n;
}

cudaError_t launch_imag_init(const double *sums, const InstDev *inst, int ii, ImagScalars *imag, cudaStream_t s)
{
    imag_init_kernel<<<1, 1, 0, s>>>(sums, inst, ii, imag);
    return cudaGetLastError();
}

__global__ void set_sigma_one_kernel(ImagScalars *__restrict__ imag, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) imag[i].sigma = 1.0;
}

cudaError_t launch_set_sigma_one(ImagScalars *imag, int n, cudaStream_t s)
{
    set_sigma_one_kernel<<<1, 128, 0, s>>>(imag, n);
    return cudaGetLastError();
}

}  // namespace gpe
