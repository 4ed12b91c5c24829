// gpe_fused.cu - the fused BCC2 half-step: Laplacian stencil (14 Hodge-weighted
// edges), potential, nonlinearity and integrator update in one pass, for every
// instance of a batch in one launch.
//
// Work decomposition: a work item is (instance, TX x TY tile of block columns,
// z-range).  A CTA of TX*TY threads owns one item at a time; thread (tx,ty)
// owns block column (x0+tx, y0+ty) and marches up the z-range.  Shared memory
// holds a ring of three z-planes of the previous field (both slots, tile plus a
// one-block halo); the plane two ahead is loaded into registers while the current
// plane is computed, so each previous-field value is read from HBM once per
// half-step (halo re-reads hit L2).  The next field is read-modified-written with
// coalesced row segments; V comes from the potential arena or per-axis trap
// tables.  Update arithmetic is gpe_device.cuh's hpsi/integrate, in the summation
// order of the BCC2 table (diagonal class first, then axial; each by dz, dy, dx).
//
// Imaginary time adds fused reductions: per thread FP32/FP64 partial sums, FP64
// across the CTA, one row per work item, and the last CTA to finish reduces each
// instance's rows in fixed order (deterministic) and updates its ImagScalars
// (next scale, mu, energy, convergence step).

#include <cuda_runtime.h>

#include "gpe_internal.h"

namespace gpe {

struct FusedArgs {
    const InstDev *__restrict__ inst;
    const WorkItem *__restrict__ items;
    int num_items;
    const void *prev;
    void *next;
    const void *vpot;
    ImagScalars *imag;
    double *partials;
    unsigned int *counter;
    const int *inst_item_begin;
    int num_instances;
    double tol;
};

template <typename T> struct Acc;      // per-thread partial sum
template <> struct Acc<double> {
    double s = 0.0;
    __device__ void add(double v) { s += v; }
    __device__ double value() const { return s; }
};
template <> struct Acc<float> {       // compensated FP32
    float s = 0.f, c = 0.f;
    __device__ void add(float v)
    {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ double value() const { return double(s) - double(c); }
};

__device__ __forceinline__ int ring_of(int zz) { return ((zz % 3) + 3) % 3; }

template <typename T, int TX, int TY, int MODE, int POT>
__global__ void __launch_bounds__(TX *TY) fused_bcc2_kernel(const FusedArgs a)
{
    using T2 = typename Cplx<T>::type;
    constexpr int NT = TX * TY;
    constexpr int PW = TX + 2, PH = TY + 2;
    constexpr int PLANE = 2 * PW * PH;
    constexpr int NLD = (PLANE + NT - 1) / NT;
    __shared__ T2 ring[3][2][PH][PW];

    const T2 *__restrict__ prev = (const T2 *)a.prev;
    T2 *__restrict__ next = (T2 *)a.next;
    const T *__restrict__ vpot = (const T *)a.vpot;
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int lx = tx + 1, ly = ty + 1;

    for (int it = blockIdx.x; it < a.num_items; it += gridDim.x) {
        const WorkItem w = a.items[it];
        const InstDev &d = a.inst[w.inst];
        const int x = w.x0 + tx, y = w.y0 + ty;
        const bool valid = (x < d.nx) && (y < d.ny);
        const T sig = (MODE == 1) ? T(a.imag[w.inst].sigma) : T(1);
        T Lw[2] = {T(d.Lc[0]), T(d.Lc[1])};
        const T L0 = T(d.L0), gdt = T(d.gdt);
        Acc<T> s0, s1, s2, s3;

        auto fetch = [&](int i, int zz) -> T2 {
            const int s = i / (PW * PH);
            const int r = i - s * (PW * PH);
            const int py = r / PW, pxl = r - py * PW;
            const int xx = w.x0 - 1 + pxl, yy = w.y0 - 1 + py;
            T2 v;
            if (xx <= d.nx && yy <= d.ny) {
                v = prev[field_index(d, s, xx, yy, zz)];
                if (MODE == 1) v = c_scale<T>(sig, v);
            } else {
                v.x = T(0);
                v.y = T(0);
            }
            return v;
        };
        auto put = [&](int i, int zz, T2 v) {
            const int s = i / (PW * PH);
            const int r = i - s * (PW * PH);
            const int py = r / PW, pxl = r - py * PW;
            ring[ring_of(zz)][s][py][pxl] = v;
        };

        // Prologue: planes z0-1, z0, z0+1 (z0+1 <= z1 <= nz, the zero plane at most).
        for (int zz = w.z0 - 1; zz <= w.z0 + 1; zz++)
            for (int i = tid; i < PLANE; i += NT) put(i, zz, fetch(i, zz));
        __syncthreads();

        for (int z = w.z0; z < w.z1; z++) {
            const bool more = (z + 2 <= w.z1);
            T2 pre[NLD];
            if (more) {
#pragma unroll
                for (int j = 0; j < NLD; j++) {
                    const int i = tid + j * NT;
                    if (i < PLANE) pre[j] = fetch(i, z + 2);
                }
            }
            if (valid) {
                const long long i0 = field_index(d, 0, x, y, z);
                const long long i1 = i0 + d.plane;
                T2 n0, n1;
                if (MODE == 0) {
                    n0 = next[i0];
                    n1 = next[i1];
                }
                T v0, v1;
                if (POT == GPE_POTENTIAL_ARRAY) {
                    v0 = vpot[i0 - d.base + d.vbase];
                    v1 = vpot[i1 - d.base + d.vbase];
                } else {
                    v0 = trap_vdt<T>(vpot, d, 0, x, y, z);
                    v1 = trap_vdt<T>(vpot, d, 1, x, y, z);
                }
                const int rm = ring_of(z - 1), r0 = ring_of(z), rp = ring_of(z + 1);
                T2 S[2];
                // slot 0 (cube corner): diagonal -> slot 1 at dz,dy,dx in {-1,0}
                S[0] = ring[rm][1][ly - 1][lx - 1];
                S[0] = c_add<T>(S[0], ring[rm][1][ly - 1][lx]);
                S[0] = c_add<T>(S[0], ring[rm][1][ly][lx - 1]);
                S[0] = c_add<T>(S[0], ring[rm][1][ly][lx]);
                S[0] = c_add<T>(S[0], ring[r0][1][ly - 1][lx - 1]);
                S[0] = c_add<T>(S[0], ring[r0][1][ly - 1][lx]);
                S[0] = c_add<T>(S[0], ring[r0][1][ly][lx - 1]);
                S[0] = c_add<T>(S[0], ring[r0][1][ly][lx]);
                // axial -> slot 0 at (dz,dy,dx) = (-1,0,0),(0,-1,0),(0,0,-1),(0,0,1),(0,1,0),(1,0,0)
                S[1] = ring[rm][0][ly][lx];
                S[1] = c_add<T>(S[1], ring[r0][0][ly - 1][lx]);
                S[1] = c_add<T>(S[1], ring[r0][0][ly][lx - 1]);
                S[1] = c_add<T>(S[1], ring[r0][0][ly][lx + 1]);
                S[1] = c_add<T>(S[1], ring[r0][0][ly + 1][lx]);
                S[1] = c_add<T>(S[1], ring[rp][0][ly][lx]);
                const T2 p0 = ring[r0][0][ly][lx];
                T hx, hy, nrm;
                hpsi<T, 2>(p0, S, Lw, L0, v0, gdt, hx, hy, nrm);
                const T2 o0 = integrate<T, MODE>(n0, p0, hx, hy);
                if (MODE == 1) {
                    s0.add(nrm);
                    s1.add(d_fma(p0.x, hx, d_mul(p0.y, hy)));
                    s2.add(d_mul(nrm, nrm));
                    s3.add(d_fma(o0.x, o0.x, d_mul(o0.y, o0.y)));
                }
                // slot 1 (cube centre): diagonal -> slot 0 at dz,dy,dx in {0,1}
                S[0] = ring[r0][0][ly][lx];
                S[0] = c_add<T>(S[0], ring[r0][0][ly][lx + 1]);
                S[0] = c_add<T>(S[0], ring[r0][0][ly + 1][lx]);
                S[0] = c_add<T>(S[0], ring[r0][0][ly + 1][lx + 1]);
                S[0] = c_add<T>(S[0], ring[rp][0][ly][lx]);
                S[0] = c_add<T>(S[0], ring[rp][0][ly][lx + 1]);
                S[0] = c_add<T>(S[0], ring[rp][0][ly + 1][lx]);
                S[0] = c_add<T>(S[0], ring[rp][0][ly + 1][lx + 1]);
                S[1] = ring[rm][1][ly][lx];
                S[1] = c_add<T>(S[1], ring[r0][1][ly - 1][lx]);
                S[1] = c_add<T>(S[1], ring[r0][1][ly][lx - 1]);
                S[1] = c_add<T>(S[1], ring[r0][1][ly][lx + 1]);
                S[1] = c_add<T>(S[1], ring[r0][1][ly + 1][lx]);
                S[1] = c_add<T>(S[1], ring[rp][1][ly][lx]);
                const T2 p1 = ring[r0][1][ly][lx];
                hpsi<T, 2>(p1, S, Lw, L0, v1, gdt, hx, hy, nrm);
                const T2 o1 = integrate<T, MODE>(n1, p1, hx, hy);
                if (MODE == 1) {
                    s0.add(nrm);
                    s1.add(d_fma(p1.x, hx, d_mul(p1.y, hy)));
                    s2.add(d_mul(nrm, nrm));
                    s3.add(d_fma(o1.x, o1.x, d_mul(o1.y, o1.y)));
                }
                next[i0] = o0;
                next[i1] = o1;
            }
            __syncthreads();
            if (more) {
#pragma unroll
                for (int j = 0; j < NLD; j++) {
                    const int i = tid + j * NT;
                    if (i < PLANE) put(i, z + 2, pre[j]);
                }
            }
            __syncthreads();
        }

        if (MODE == 1) {
            // CTA reduction of the four sums in FP64, fixed shape.
            double v[4] = {s0.value(), s1.value(), s2.value(), s3.value()};
#pragma unroll
            for (int k = 0; k < 4; k++)
                for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
            __shared__ double red[NT / 32][4];
            const int warp = tid >> 5, lane = tid & 31;
            if (lane == 0)
                for (int k = 0; k < 4; k++) red[warp][k] = v[k];
            __syncthreads();
            if (tid < 4) {
                double t = 0.0;
                for (int wi = 0; wi < NT / 32; wi++) t += red[wi][tid];
                a.partials[4ll * it + tid] = t;
            }
            __syncthreads();
        }
    }

    if (MODE == 1) {
        // Last CTA to finish reduces every instance's rows (fixed order) and
        // updates its imaginary-time scalars.
        __shared__ bool last;
        __threadfence();
        __syncthreads();
        if (tid == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
        __syncthreads();
        if (!last) return;
        __threadfence();
        const int warp = tid >> 5, lane = tid & 31;
        for (int i = warp; i < a.num_instances; i += NT / 32) {
            const int b = a.inst_item_begin[2 * i], e = a.inst_item_begin[2 * i + 1];
            double acc[4];
            for (int k = 0; k < 4; k++) {
                double s = 0.0, c = 0.0;
                for (int r = b + lane; r < e; r += 32) {
                    const double yv = __ldcg(a.partials + 4ll * r + k) - c;
                    const double t = s + yv;
                    c = (t - s) - yv;
                    s = t;
                }
                for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
                acc[k] = s;
            }
            if (lane == 0) {
                const InstDev &d = a.inst[i];
                ImagScalars &st = a.imag[i];
                // acc: |p'|^2, Re(conj(p') dt H p'), |p'|^4, |next|^2 over values
                const double nin = d.vol * acc[0];
                const double mu = acc[1] / (d.dt * acc[0]);
                st.norm_in = nin;
                st.energy = d.vol * (acc[1] / d.dt - 0.5 * d.g * acc[2]);
                st.mu_prev = st.mu;
                st.mu = mu;
                st.dmu = (st.steps > 0) ? fabs(mu - st.mu_prev) : INFINITY;
                if (st.steps > 0 && st.conv_step < 0 && st.dmu < a.tol) st.conv_step = st.steps;
                st.steps += 1;
                st.sigma = 1.0 / sqrt(d.vol * acc[3]);
            }
        }
        if (tid == 0) *a.counter = 0u;
    }
}

// Tile variants (TX, TY).  Index 0 is the default.
static const int kTiles[][2] = {{32, 8}, {32, 4}, {16, 16}, {16, 8}, {64, 4}, {8, 32}};

int fused_tile_count() { return int(sizeof(kTiles) / sizeof(kTiles[0])); }
void fused_tile_shape(int tile, int *tx, int *ty)
{
    if (tile < 0 || tile >= fused_tile_count()) tile = 0;
    *tx = kTiles[tile][0];
    *ty = kTiles[tile][1];
}

template <typename T, int TX, int TY>
static cudaError_t fused_launch_t(const FusedLaunch &l, const FusedArgs &a, cudaStream_t s)
{
    const int g = l.grid;
    if (l.mode == GPE_REAL_TIME) {
        if (l.potential == GPE_POTENTIAL_ARRAY) fused_bcc2_kernel<T, TX, TY, 0, 0><<<g, TX * TY, 0, s>>>(a);
        else fused_bcc2_kernel<T, TX, TY, 0, 1><<<g, TX * TY, 0, s>>>(a);
    } else {
        if (l.potential == GPE_POTENTIAL_ARRAY) fused_bcc2_kernel<T, TX, TY, 1, 0><<<g, TX * TY, 0, s>>>(a);
        else fused_bcc2_kernel<T, TX, TY, 1, 1><<<g, TX * TY, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <typename T>
static cudaError_t fused_launch_tile(const FusedLaunch &l, const FusedArgs &a, cudaStream_t s)
{
    switch (l.tile) {
    case 1: return fused_launch_t<T, 32, 4>(l, a, s);
    case 2: return fused_launch_t<T, 16, 16>(l, a, s);
    case 3: return fused_launch_t<T, 16, 8>(l, a, s);
    case 4: return fused_launch_t<T, 64, 4>(l, a, s);
    case 5: return fused_launch_t<T, 8, 32>(l, a, s);
    default: return fused_launch_t<T, 32, 8>(l, a, s);
    }
}

cudaError_t launch_fused_step(const FusedLaunch &l, cudaStream_t s)
{
    FusedArgs a;
    a.inst = l.inst;
    a.items = l.items;
    a.num_items = l.num_items;
    a.prev = l.prev;
    a.next = l.next;
    a.vpot = l.vpot;
    a.imag = l.imag;
    a.partials = l.partials;
    a.counter = l.counter;
    a.inst_item_begin = l.inst_item_begin;
    a.num_instances = l.num_instances;
    a.tol = l.tol;
    if (l.precision == GPE_FP64) return fused_launch_tile<double>(l, a, s);
    return fused_launch_tile<float>(l, a, s);
}

}  // namespace gpe
