// gpe_fused_t12.cu - the fused half-step for the TETRA12 lattice (the
// reference's own discretisation: 12 values per block, 4 neighbours each) in
// FP32: the same update as the plain kernel, fed by a TMA ring of planes.  The
// lattice form is the reference's update (GPUGrossPitaevskii_BCC.cu:176-216, its
// neighbour order); the face form is its multi-GPU program's Hodge form
// (GPUGrossPitaevskii_BCC_multi.cu:329-397, faces and weights from the handle).
// Real time (MODE 0) or imaginary time (MODE 1: the previous field scaled by
// sigma as it is read, the item's sums folded at the end of the grid).
//
// One CTA runs one work item (instance, TX x TY tile of block columns, z-range).
// The producer lane loads, per plane q = z0-1 .. z1, the previous field's box of
// all 12 slots over the tile plus a 2-column / 1-row halo, and with it the next
// field's interior tile of plane q-1.  A value's neighbours lie within one block
// in x, y and z, so output plane z needs the previous field's planes z-1, z and
// z+1: the ring keeps three planes resident while the producer runs ahead by
// STAGES - 3.  Consumer warp w handles slot w for the tile's 32 columns, row
// after row, so every table lookup is uniform across the warp; the sums follow
// the table order exactly as the plain kernel's do, so the two kernels' results
// are the same bit for bit in real time.  Every mbarrier wait is bounded (about
// a second); a timeout sets the launch's error word and the CTA returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include "gpe_fused_core.cuh"

namespace gpe {

template <int TX, int TY, int POT>
struct T12Shape {
    static constexpr int NS = 12;
    static constexpr int BW = TX + 4;                    // x0-2 .. x0+TX+1
    static constexpr int BH = TY + 2;                    // y0-1 .. y0+TY
    static constexpr int PREV_SLOT = BW * BH;            // float2 per slot in the halo box
    static constexpr int PREV_BYTES = NS * PREV_SLOT * 8;
    static constexpr int NEXT_SLOT = TX * TY;
    static constexpr int NEXT_BYTES = NS * NEXT_SLOT * 8;
    static constexpr int NEXT_OFF = ((PREV_BYTES + 127) / 128) * 128;
    // ARRAY potential: L0 + V dt of the next tile's plane, columns x0-2 .. x0+TX+1
    // (a 16-byte-aligned box of 4-byte values), TY rows, all slots
    static constexpr int V_SLOT = BW * TY;
    static constexpr int V_BYTES = POT == GPE_POTENTIAL_ARRAY ? NS * V_SLOT * 4 : 0;
    static constexpr int V_OFF = ((NEXT_OFF + NEXT_BYTES + 127) / 128) * 128;
    static constexpr int STAGE_BYTES = ((V_OFF + V_BYTES + 127) / 128) * 128;
    static constexpr int NCONS = NS * 32;                // one consumer warp per slot
    static constexpr int NTHREADS = NCONS + 32;          // plus the producer warp
};

template <int TX, int TY, int POT, int STAGES>
int t12_smem_bytes()
{
    return STAGES * T12Shape<TX, TY, POT>::STAGE_BYTES + 128 + 16 * STAGES;
}

struct T12Args {
    const InstDev *__restrict__ inst;
    ImagScalars *imag;        // imaginary time: per-instance scalars (sigma in, sums folded out)
    double *partials;         // imaginary time: 4 sums per work item
    unsigned int *counter;    // imaginary time: CTAs done
    const int *inst_item_begin;
    int num_instances;
    double tol;
    const WorkItem *__restrict__ items;
    const CUtensorMap *maps;  // [instance][field][prev box, next box]
    const CUtensorMap *vmaps; // ARRAY potential: [instance] (L0 + V dt, next-tile box)
    int src;                  // field index of prev
    float2 *next;
    const float *vpot;        // TRAP: per-axis tables; ARRAY: L0 + V dt per value
    int *err;
    int inject_skip_plane;
    int tab[48];              // packed neighbour entries, slot-major, the reference's order
};

template <int TX, int TY, int MODE, int POT, int STAGES, bool FACE>
__global__ void __launch_bounds__(T12Shape<TX, TY, POT>::NTHREADS, 1) fused_t12_kernel(const T12Args a)
{
    static_assert(TX == 32, "one lane per column of the tile");
    static_assert(STAGES >= 4, "three resident planes and one in flight");
    using S = T12Shape<TX, TY, POT>;
    constexpr bool REAL = MODE == 0;  // MODE 1: imaginary time (psi' = sigma psi - dt H sigma psi)
    constexpr int NWARPS = S::NTHREADS / 32;
    extern __shared__ unsigned char dyn_smem[];
    const uint32_t raw = smem_u32(dyn_smem);
    const uint32_t base = (raw + 127u) & ~127u;
    unsigned char *const gbase = dyn_smem + (base - raw);
    const uint32_t full = base + STAGES * S::STAGE_BYTES;
    const uint32_t empty = full + 8 * STAGES;
    __shared__ volatile int abort_flag;
    __shared__ double row_sums[4];  // imaginary time: this work item's four sums

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const WorkItem w = a.items[blockIdx.x];
    const InstDev &d = a.inst[w.inst];
    const int nplanes = w.z1 - w.z0 + 2;  // previous-field planes z0-1 .. z1

    if (tid == 0) {
        abort_flag = 0;
        for (int st = 0; st < STAGES; st++) {
            mbar_init(full + 8 * st, 1);
            mbar_init(empty + 8 * st, S::NS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    grid_dependency_wait();
    __syncthreads();

    if (warp == S::NS) {
        // ---- producer lane ----------------------------------------------------
        if (lane == 0) {
            const CUtensorMap *prevmap = a.maps + 4 * w.inst + 2 * a.src;
            const CUtensorMap *nextmap = a.maps + 4 * w.inst + 2 * (1 - a.src) + 1;
            int issued = 0;
            for (int k = 0; k < nplanes; k++) {
                const int st = k % STAGES;
                if (k >= STAGES) {
                    const uint32_t par = ((k / STAGES) - 1) & 1;
                    bool ok = mbar_try_wait(empty + 8 * st, par);
                    const uint64_t t0 = global_ns();
                    while (!ok && !*(volatile int *)&abort_flag && global_ns() - t0 <= kWaitLimitNs)
                        ok = mbar_try_wait(empty + 8 * st, par);
                    if (!ok) {
                        atomicExch(a.err, kErrTimeout);
                        abort_flag = 1;
                        break;
                    }
                }
                if (a.inject_skip_plane == k && blockIdx.x == 0) break;  // test hook: withhold this plane
                const bool with_next = k >= 2;
                mbar_arrive_expect_tx(full + 8 * st,
                                      S::PREV_BYTES + (with_next ? (REAL ? S::NEXT_BYTES : 0) + S::V_BYTES : 0));
                // padded coordinates: x0-2 -> x0-2+kPadX, y0-1 -> y0, plane q -> q+1
                tma_load_4d(base + st * S::STAGE_BYTES, prevmap, w.x0 - 2 + kPadX, w.y0, 0, w.z0 + k, full + 8 * st);
                if (REAL && with_next)  // next field, interior tile of plane q-1
                    tma_load_4d(base + st * S::STAGE_BYTES + S::NEXT_OFF, nextmap, w.x0 + kPadX, w.y0 + 1, 0,
                                w.z0 + k - 1, full + 8 * st);
                if (POT == GPE_POTENTIAL_ARRAY && with_next)  // and its L0 + V dt
                    tma_load_4d(base + st * S::STAGE_BYTES + S::V_OFF, a.vmaps + w.inst, w.x0 - 2 + kPadX, w.y0 + 1, 0,
                                w.z0 + k - 1, full + 8 * st);
                issued = k + 1;
            }
            if (abort_flag) drain_ring<STAGES>(issued, full);
        }
    } else {
        Acc<float> acc[4];  // imaginary time: |p|^2, Re(conj(p) h), |p|^4, |next|^2
        // ---- consumer warp: slot s, columns x0 .. x0+31 --------------------------
        const int s = warp;
        const int x = w.x0 + lane;
        const bool xin = x < d.nx;
        const float Lw[1] = {float(d.Lc[0])};
        const float L0 = float(d.L0), gdt = float(d.gdt);
        // trap: Vx + Vy of the thread's column and rows, Vz per plane
        float vxy[TY];
        const float *tz = nullptr;
        if (POT == GPE_POTENTIAL_TRAP) {
            const float *txt = a.vpot + d.vbase;
            const float *tyt = txt + (long long)d.slots * d.nx;
            tz = tyt + (long long)d.slots * d.ny;
            const float vx = xin ? txt[s * d.nx + x] : 0.f;
#pragma unroll
            for (int ty = 0; ty < TY; ty++) vxy[ty] = w.y0 + ty < d.ny ? d_add(vx, tyt[s * d.ny + w.y0 + ty]) : 0.f;
        }
        int off[4], dzk[4];  // per neighbour: offset in its plane's box, plane (-1, 0, +1)
        float hk[4];         // FACE: the faces' weights -0.5 hodge / bs^2 * dt, summation order
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int e = FACE ? d.fe[4 * s + k] : a.tab[s * 4 + k];
            hk[k] = FACE ? d.hf32[4 * s + k] : 0.f;
            const int dx = (e & 3) - 1, dy = ((e >> 2) & 3) - 1, dz = ((e >> 4) & 3) - 1, sl = (e >> 6) & 15;
            off[k] = sl * S::PREV_SLOT + (1 + dy) * S::BW + (lane + 2 + dx);
            dzk[k] = dz;
        }
        const int selfoff = s * S::PREV_SLOT + S::BW + lane + 2;
        const float sig = (MODE == 1) ? float(a.imag[w.inst].sigma) : 1.f;
        for (int k = 0; k < nplanes; k++) {
            const int st = k % STAGES;
            const bool got = mbar_wait_bounded(full + 8 * st, (k / STAGES) & 1);
            if (__any_sync(0xffffffffu, !got)) {
                if (lane == 0) {
                    atomicExch(a.err, kErrTimeout);
                    abort_flag = 1;
                }
                break;
            }
            if (k < 2) continue;
            const int z = w.z0 - 2 + k;  // output plane: previous planes z-1, z, z+1 in stages k-2, k-1, k
            const float2 *Pm = (const float2 *)(gbase + ((k - 2) % STAGES) * S::STAGE_BYTES);
            const float2 *P0 = (const float2 *)(gbase + ((k - 1) % STAGES) * S::STAGE_BYTES);
            const float2 *Pp = (const float2 *)(gbase + st * S::STAGE_BYTES);
            const float2 *N = (const float2 *)(gbase + st * S::STAGE_BYTES + S::NEXT_OFF) + s * S::NEXT_SLOT + lane;
            const float *Vb = (const float *)(gbase + st * S::STAGE_BYTES + S::V_OFF) + s * S::V_SLOT + lane + 2;
            const float2 *Q[4];
#pragma unroll
            for (int kk = 0; kk < 4; kk++) Q[kk] = (dzk[kk] < 0 ? Pm : (dzk[kk] > 0 ? Pp : P0)) + off[kk];
            const float vz = (POT == GPE_POTENTIAL_TRAP) ? tz[s * d.nz + z] : 0.f;
#pragma unroll
            for (int ty = 0; ty < TY; ty++) {
                const int y = w.y0 + ty;
                const int r = ty * S::BW;
                auto rd = [&](float2 v) { return MODE == 1 ? c_scale<float>(sig, v) : v; };
                const float2 p = rd(P0[selfoff + r]);
                float2 Sg[1];
                float fx = 0.f, fy = 0.f;  // FACE: sum of h_k (psi_k - psi), one fma per face
                if (FACE) {
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const float2 v = rd(Q[kk][r]);
                        fx = d_fma(hk[kk], d_sub(v.x, p.x), fx);
                        fy = d_fma(hk[kk], d_sub(v.y, p.y), fy);
                    }
                } else {
                    Sg[0] = rd(Q[0][r]);
#pragma unroll
                    for (int kk = 1; kk < 4; kk++) Sg[0] = c_add<float>(Sg[0], rd(Q[kk][r]));
                }
                const float2 n = REAL ? N[ty * TX] : make_float2(0.f, 0.f);
                if (xin && y < d.ny) {
                    const long long self = field_index(d, s, x, y, z);
                    float hx, hy, nrm;
                    if (FACE) {
                        // the face form's update (the multi-GPU program's roundings):
                        // c = fma(g dt, fma(x, x, y y), V dt), h = fma(c, psi, sum)
                        const float vdt = POT == GPE_POTENTIAL_ARRAY ? Vb[ty * S::BW] : d_add(vxy[ty], vz);
                        nrm = d_fma(p.x, p.x, d_mul(p.y, p.y));
                        const float c = d_fma(gdt, nrm, vdt);
                        hx = d_fma(c, p.x, fx);
                        hy = d_fma(c, p.y, fy);
                    } else if (POT == GPE_POTENTIAL_ARRAY) {
                        hpsi<float, 1, true>(p, Sg, Lw, L0, Vb[ty * S::BW], gdt, hx, hy, nrm);
                    } else {
                        const float vdt = d_add(vxy[ty], vz);
                        hpsi<float, 1, false>(p, Sg, Lw, L0, vdt, gdt, hx, hy, nrm);
                    }
                    const float2 o = integrate<float, MODE>(n, p, hx, hy);
                    a.next[self] = o;
                    if (MODE == 1) {
                        acc[0].add(nrm);
                        acc[1].add(d_fma(p.x, hx, d_mul(p.y, hy)));
                        acc[2].add(d_mul(nrm, nrm));
                        acc[3].add(d_fma(o.x, o.x, d_mul(o.y, o.y)));
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + 8 * ((k - 2) % STAGES));  // plane z-1 is no longer read
        }
        if (MODE == 1) {
            double v[4] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
#pragma unroll
            for (int k = 0; k < 4; k++)
                for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
            __shared__ double red[S::NS][4];
            if (lane == 0)
                for (int k = 0; k < 4; k++) red[warp][k] = v[k];
            asm volatile("bar.sync 1, %0;" ::"r"(S::NCONS) : "memory");  // consumer warps only
            if (tid < 4) {
                double t = 0.0;
                for (int wi = 0; wi < S::NS; wi++) t += red[wi][tid];
                row_sums[tid] = t;
            }
        }
    }
    launch_dependents();
    if (MODE == 1)
        imag_publish_and_fold<NWARPS>(blockIdx.x, row_sums, abort_flag, S::NS, a.partials, a.counter,
                                      a.inst_item_begin, a.num_instances, a.inst, a.imag, a.tol);
}

// Variants: tile (TX, TY) and pipeline depth.  The first four run one CTA per SM
// (the largest ring, 32 x 6 with 5 stages, takes 230,608 of the 232,448 bytes a
// CTA may have); the last two fit two CTAs per SM with the trap potential.
struct T12Variant {
    int tx, ty, stages;
};
static const T12Variant kT12Variants[] = {{32, 4, 6}, {32, 2, 8}, {32, 6, 5}, {32, 3, 7}, {32, 2, 5}, {32, 3, 4}};
constexpr int kT12Count = int(sizeof(kT12Variants) / sizeof(kT12Variants[0]));

int t12_variant_count() { return kT12Count; }
void t12_variant(int v, int *tx, int *ty, int *stages)
{
    if (v < 0 || v >= kT12Count) v = 0;
    *tx = kT12Variants[v].tx;
    *ty = kT12Variants[v].ty;
    *stages = kT12Variants[v].stages;
}

template <int TX, int TY, int MODE, int POT, int STAGES, bool FACE>
static cudaError_t launch_t12_t(const T12Args &a, int grid, cudaStream_t s)
{
    const int bytes = t12_smem_bytes<TX, TY, POT, STAGES>();
    auto kern = fused_t12_kernel<TX, TY, MODE, POT, STAGES, FACE>;
    static int allowed = 48 * 1024;
    if (bytes > allowed) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        allowed = bytes;
    }
    // Real time: programmatic dependent launch.  Imaginary time ends every grid
    // with the fold in its last CTA; an early-scheduled next grid there would
    // only hold SM slots, so it launches plainly.
    if (MODE == 0) return launch_pdl(kern, grid, T12Shape<TX, TY, POT>::NTHREADS, bytes, s, a);
    kern<<<grid, T12Shape<TX, TY, POT>::NTHREADS, bytes, s>>>(a);
    return cudaGetLastError();
}

// With an ARRAY potential each stage also holds the L0 + V dt box, so the
// deeper variants give up a stage to stay within the CTA's shared memory.
template <int MODE, int POT, bool FACE>
static cudaError_t launch_t12_pot(int variant, const T12Args &a, int grid, cudaStream_t s)
{
    constexpr bool A = POT == GPE_POTENTIAL_ARRAY;
    switch (variant) {  // must list kT12Variants in order
    case 1: return launch_t12_t<32, 2, MODE, POT, 8, FACE>(a, grid, s);
    case 2: return launch_t12_t<32, 6, MODE, POT, A ? 4 : 5, FACE>(a, grid, s);
    case 3: return launch_t12_t<32, 3, MODE, POT, 7, FACE>(a, grid, s);
    case 4: return launch_t12_t<32, 2, MODE, POT, A ? 4 : 5, FACE>(a, grid, s);
    case 5: return launch_t12_t<32, 3, MODE, POT, 4, FACE>(a, grid, s);
    default: return launch_t12_t<32, 4, MODE, POT, A ? 5 : 6, FACE>(a, grid, s);
    }
}

template <int MODE, int POT>
static cudaError_t launch_t12_form(bool face, int variant, const T12Args &a, int grid, cudaStream_t s)
{
    if (face) return launch_t12_pot<MODE, POT, true>(variant, a, grid, s);
    return launch_t12_pot<MODE, POT, false>(variant, a, grid, s);
}

cudaError_t launch_t12_step(const T12Launch &l, cudaStream_t s)
{
    T12Args a;
    a.inst = l.inst;
    a.imag = l.imag;
    a.partials = l.partials;
    a.counter = l.counter;
    a.inst_item_begin = l.inst_item_begin;
    a.num_instances = l.num_instances;
    a.tol = l.tol;
    a.items = l.items;
    a.maps = (const CUtensorMap *)l.maps;
    a.vmaps = (const CUtensorMap *)l.vmaps;
    a.src = l.src;
    a.next = (float2 *)l.next;
    a.vpot = (const float *)l.vpot;
    a.err = l.err;
    a.inject_skip_plane = l.inject_skip_plane;
    for (int i = 0; i < 48; i++) a.tab[i] = l.tab[i];
    const bool arr = l.potential == GPE_POTENTIAL_ARRAY;
    if (l.mode == GPE_IMAGINARY_TIME) {
        if (arr) return launch_t12_form<1, GPE_POTENTIAL_ARRAY>(l.face, l.variant, a, l.grid, s);
        return launch_t12_form<1, GPE_POTENTIAL_TRAP>(l.face, l.variant, a, l.grid, s);
    }
    if (arr) return launch_t12_form<0, GPE_POTENTIAL_ARRAY>(l.face, l.variant, a, l.grid, s);
    return launch_t12_form<0, GPE_POTENTIAL_TRAP>(l.face, l.variant, a, l.grid, s);
}

}  // namespace gpe
