// gpe_fused.cu - the fused BCC2 half-step: Laplacian stencil (14 Hodge-weighted
// edges), potential, nonlinearity and integrator update in one pass, for every
// instance of a batch in one launch.
//
// Work decomposition: a work item is (instance, TX x TY tile of block columns,
// z-range [z0, z1)); one CTA of TX*TY threads per item; thread (tx, ty) owns
// block column (x0+tx, y0+ty) and marches up z.
//
// Data movement (sm_103a), warp-specialised:
//  * One producer warp issues TMA copies into a STAGES-deep shared-memory ring:
//    for every plane q in [z0-1, z1] a cp.async.bulk.tensor 4-D copy brings the
//    previous field's tile plus halo (x0-2 .. x0+TX+1 so that the copy starts
//    on a 16-byte boundary, y0-1 .. y0+TY, both slots), and in the same stage
//    the next field's interior tile of plane q-1 (read-modify-write input).
//    Each stage has a "full" mbarrier (transaction bytes) and an "empty"
//    mbarrier (one arrival per consumer warp); the producer refills a stage
//    once every consumer warp has released it, so warps never wait for each
//    other at a CTA-wide barrier and up to STAGES planes are in flight.
//  * Each consumer thread reads a plane from shared memory once (12 values of
//    its 3x3 neighbourhood, both slots, plus its next-field values) and carries
//    what later planes need in registers: its own values of the previous two
//    planes, the pending diagonal sum and box sum, the in-plane axial sums.
//  * Results are stored with coalesced row writes straight from registers.
//    The trap potential's z-term of the CTA's z-range is staged in shared
//    memory once; an array potential is read with plain loads.
//
// Summation order (the oracle's oracle_half_step_bcc2_* mirrors it bit for bit),
// with C = slot 0 (cube corner), B = slot 1 (cube centre):
//   bB(q) = (B(x-1,y-1) + B(x,y-1)) + (B(x-1,y) + B(x,y))      at plane q
//   bC(q) = (C(x,y) + C(x+1,y)) + (C(x,y+1) + C(x+1,y+1))      at plane q
//   slot 0 at z: Sd = bB(z-1) + bB(z), Sa = (C(z-1) + C(z+1)) + ((C(x-1) + C(x+1)) + (C(y-1) + C(y+1)))
//   slot 1 at z: Sd = bC(z) + bC(z+1), Sa = (B(z-1) + B(z+1)) + ((B(x-1) + B(x+1)) + (B(y-1) + B(y+1)))
// followed by gpe_device.cuh's hpsi/integrate (the reference's update,
// GPUGrossPitaevskii_BCC.cu:207-215).
//
// Every mbarrier wait is bounded; on timeout the CTA records an error code,
// waits (bounded) for its own copies in flight, and returns.
//
// Imaginary time adds fused reductions: per-thread compensated sums, FP64
// across the CTA, one row per work item; the last CTA to finish reduces each
// instance's rows in fixed order and updates its ImagScalars.
//
// Compensated real time (MODE 2, FP32 only): every value of the next field also
// carries an int8 residual per component in units of the stored component's
// ulp / 256 (one 16-bit word, same padded index as the field; gpe_device.cuh).
// The update adds the residual to the increment, adds that to the stored value
// with an exact two-sum, and stores the rounded sum and its rounding error in
// those units:
//   t = lo + (hy, -hx);  s = n + t;  b = s - n;  r = (n - (s - b)) + (t - b)
// so the time accumulation keeps about 8 more bits than FP32 storage.  The
// residual tile travels by TMA in the same stage as the next field's tile (TMA
// reads L2; plain loads through L1 saw stale residuals when consecutive grids
// overlapped under programmatic dependent launch); results are stored from
// registers.

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>

#include <string>

#include "gpe_fused_core.cuh"
#include "gpe_internal.h"

namespace gpe {

struct FusedArgs {
    const InstDev *__restrict__ inst;
    const WorkItem *__restrict__ items;
    int num_items;
    const CUtensorMap *maps;  // [instance][field][halo box, interior box]
    const CUtensorMap *lo_maps;  // MODE 2: [instance][field] residual box
    int zcmax;                // longest z-range of a work item
    int src;                  // field the previous values come from (0 or 1)
    const void *prev;
    void *next;
    uint16_t *next_lo;        // MODE 2: int8 x 2 residuals of the next field
    const void *vpot;
    ImagScalars *imag;
    double *partials;
    unsigned int *counter;
    const int *inst_item_begin;
    int num_instances;
    double tol;
    int *err;
    int inject_skip_plane;  // test hook: plane the producer of work item 0 withholds (-1 = none)
};

template <typename T, int TX, int TY, int MODE, int POT, int STAGES, int MINB>
__global__ void __launch_bounds__(TX *TY + 32, MinBlocks<T, MINB>::value) fused_bcc2_kernel(const FusedArgs a)
{
    static_assert(MODE != 2 || sizeof(T) == 4, "compensated storage is an FP32 mode");
    constexpr bool REAL = MODE != 1;  // MODE 0 and 2 advance real time
    using S = FusedShape<T, TX, TY, MODE == 2>;
    using T2 = typename S::T2;
    constexpr int NT = S::NT;
    constexpr int NWARPS = S::NTHREADS / 32;
    extern __shared__ unsigned char dyn_smem[];
    const uint32_t raw = smem_u32(dyn_smem);
    const uint32_t base = (raw + 127u) & ~127u;
    unsigned char *const gbase = dyn_smem + (base - raw);
    const uint32_t full = base + STAGES * S::STAGE_BYTES;
    const uint32_t empty = full + 8 * STAGES;
    T *const ztab = (T *)(gbase + STAGES * S::STAGE_BYTES + 16 * STAGES);
    __shared__ volatile int abort_flag;
    __shared__ double row_sums[4];  // imaginary time: this work item's four sums

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int it = blockIdx.x;
    const WorkItem w = a.items[it];
    const InstDev &d = a.inst[w.inst];
    const int nz = d.nz;

    if (tid == 0) {
        abort_flag = 0;
        for (int st = 0; st < STAGES; st++) {
            mbar_init(full + 8 * st, 1);
            mbar_init(empty + 8 * st, NT / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (POT == GPE_POTENTIAL_TRAP) {
        // z-term of the trap for this item's z-range, both slots
        const T *tz = (const T *)a.vpot + d.vbase + 2ll * d.nx + 2ll * d.ny;
        const int zl = w.z1 - w.z0;
        for (int i = tid; i < 2 * zl; i += S::NTHREADS) {
            const int sl = i / zl, z = w.z0 + (i - sl * zl);
            ztab[i] = tz[sl * nz + z];
        }
    }
    // Programmatic dependent launch: this grid may start while the previous one
    // drains; nothing it wrote (fields, imaginary-time scalars) is read before here.
    grid_dependency_wait();
    __syncthreads();

    if (warp == NWARPS - 1) {
        // ---- producer warp ------------------------------------------------
        if (lane == 0) {
            int issued = 0;
            produce_item<T, TX, TY, MODE, STAGES, false>(w, 0, a.src, a.maps, a.lo_maps, base, full, empty,
                                                        it == 0 ? a.inject_skip_plane : -1, a.err, &abort_flag,
                                                        issued);
            if (abort_flag) drain_ring<STAGES>(issued, full);  // let this CTA's copies land before it exits
        }
    } else {
        // ---- consumer warps ----------------------------------------------
        const T sig = (MODE == 1) ? T(a.imag[w.inst].sigma) : T(1);
        Acc<T> acc[4];
        consume_item<T, TX, TY, MODE, POT, STAGES, false>(w, d, 0, gbase, full, empty, a.next, a.next_lo, a.vpot,
                                                          ztab, w.z1 - w.z0, w.z0, sig, acc, tid, lane, a.err,
                                                          &abort_flag);
        Acc<T> &s0 = acc[0], &s1 = acc[1], &s2 = acc[2], &s3 = acc[3];
        if (MODE == 1) {
            double v[4] = {s0.value(), s1.value(), s2.value(), s3.value()};
#pragma unroll
            for (int k = 0; k < 4; k++)
                for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
            __shared__ double red[NT / 32][4];
            if (lane == 0)
                for (int k = 0; k < 4; k++) red[warp][k] = v[k];
            asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");  // consumer warps only
            if (tid < 4) {
                double t = 0.0;
                for (int wi = 0; wi < NT / 32; wi++) t += red[wi][tid];
                row_sums[tid] = t;
            }
        }
    }

    launch_dependents();  // the next grid may be scheduled; it waits for this one to finish
    if (MODE == 1)
        imag_publish_and_fold<NWARPS>(it, row_sums, abort_flag, NWARPS - 1, a.partials, a.counter,
                                      a.inst_item_begin, a.num_instances, a.inst, a.imag, a.tol);
}

// ---- Both half-steps of a leapfrog step in one pass --------------------------
// Reads the even field E and odd field O of one buffer set and writes
// O' = O - i H(E) and E' = E - i H(O') into the other set, so each step moves
// 32 instead of 48 bytes per vertex (FP32).  Per work item (tile TX x TY of
// one instance, planes z0..z1-1) the consumer threads cover the tile plus a
// one-block ring, (TX+2) x (TY+2) columns:
//   phase A  every thread computes O'(p) of its column from the E stencil (E box:
//            tile plus a 2-block ring) and O(p) (O box: tile plus a 1-block
//            ring), exactly as the one-half-step kernel does, and leaves O'(p)
//            in a shared plane buffer; O' is zero outside the instance;
//   phase B  after a barrier of the consumer warps the tile's threads compute
//            E'(p-1) from the O' stencil in that buffer and their own E(p-1)
//            carried from phase A.
// Planes z0-1 and z1 of O' are computed again here (the neighbouring items
// compute them too) so that no CTA waits for another.  The sums follow the
// same order as the one-half-step kernel, so the result is bit-identical to two
// of its launches.
template <typename T, int TX, int TY>
struct TwoStepShape {
    using T2 = typename Cplx<T>::type;
    static constexpr int EX = TX + 2, EY = TY + 2;  // thread box
    static constexpr int NT = ((EX * EY + 31) / 32) * 32;
    static constexpr int NTHREADS = NT + 32;
    static constexpr int BW = TX + 4;  // box columns x0-2 .. x0+TX+1
    static constexpr int EH = TY + 4;  // E box rows y0-2 .. y0+TY+1
    static constexpr int OH = TY + 2;  // O box rows y0-1 .. y0+TY
    static constexpr int E_BYTES = 2 * BW * EH * (int)sizeof(T2);
    static constexpr int O_BYTES = 2 * BW * OH * (int)sizeof(T2);
    static constexpr int O_OFF = ((E_BYTES + 127) / 128) * 128;
    static constexpr int STAGE_BYTES = ((O_OFF + O_BYTES + 127) / 128) * 128;
    static constexpr int NEW_SLOT = EX * EY;
    static constexpr int NEW_BYTES = ((2 * NEW_SLOT * (int)sizeof(T2) + 127) / 128) * 128;
    static constexpr int XE = (int)sizeof(T2) / 8;
};

template <typename T, int TX, int TY, int STAGES>
int twostep_smem_bytes(int zcmax)
{
    using S = TwoStepShape<T, TX, TY>;
    return STAGES * S::STAGE_BYTES + 2 * S::NEW_BYTES + 128 + 16 * STAGES + 2 * (zcmax + 2) * (int)sizeof(T) + 16;
}

struct TwoStepArgs {
    const InstDev *__restrict__ inst;
    const WorkItem *__restrict__ items;
    const CUtensorMap *maps;  // [instance][set][E box, O box]
    int set;                  // buffer set read (0 or 1)
    int zcmax;
    void *out_e, *out_o;      // field arenas of the other set
    const void *vpot;
    int *err;
    int inject_skip_plane;
};

template <typename T, int TX, int TY, int POT, int STAGES, int MINB>
__global__ void __launch_bounds__(TwoStepShape<T, TX, TY>::NTHREADS, MinBlocks<T, MINB>::value)
    twostep_bcc2_kernel(const TwoStepArgs a)
{
    using S = TwoStepShape<T, TX, TY>;
    using T2 = typename S::T2;
    constexpr int NT = S::NT;
    constexpr int NWARPS = S::NTHREADS / 32;
    extern __shared__ unsigned char dyn_smem[];
    const uint32_t raw = smem_u32(dyn_smem);
    const uint32_t base = (raw + 127u) & ~127u;
    unsigned char *const gbase = dyn_smem + (base - raw);
    T2 *const newbuf = (T2 *)(gbase + STAGES * S::STAGE_BYTES);  // two O' planes
    const uint32_t full = base + STAGES * S::STAGE_BYTES + 2 * S::NEW_BYTES;
    const uint32_t empty = full + 8 * STAGES;
    T *const ztab = (T *)(gbase + STAGES * S::STAGE_BYTES + 2 * S::NEW_BYTES + 16 * STAGES);
    __shared__ int abort_flag;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int it = blockIdx.x;
    const WorkItem w = a.items[it];
    const InstDev &d = a.inst[w.inst];
    const int zl = w.z1 - w.z0;
    const int nplanes = zl + 4;  // E planes z0-2 .. z1+1
    const int nz = d.nz;

    if (tid == 0) {
        abort_flag = 0;
        for (int st = 0; st < STAGES; st++) {
            mbar_init(full + 8 * st, 1);
            mbar_init(empty + 8 * st, NT / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (POT == GPE_POTENTIAL_TRAP) {
        // z-term of the trap for planes z0-1 .. z1 (clamped into the instance), both slots
        const T *tz = (const T *)a.vpot + d.vbase + 2ll * d.nx + 2ll * d.ny;
        const int zn = zl + 2;
        for (int i = tid; i < 2 * zn; i += S::NTHREADS) {
            const int sl = i / zn;
            const int z = min(max(w.z0 - 1 + (i - sl * zn), 0), nz - 1);
            ztab[i] = tz[sl * nz + z];
        }
    }
    grid_dependency_wait();
    __syncthreads();

    if (warp == NWARPS - 1) {
        // ---- producer warp: E(q) and O(q-1) for q = z0-2 .. z1+1 -------------
        if (lane == 0) {
            const CUtensorMap *emap = a.maps + 4 * w.inst + 2 * a.set;
            const CUtensorMap *omap = emap + 1;
            int issued = 0;
            for (int k = 0; k < nplanes; k++) {
                const int st = k % STAGES;
                if (k >= STAGES) {
                    bool ok = mbar_try_wait(empty + 8 * st, ((k / STAGES) - 1) & 1);
                    const uint64_t t0 = global_ns();
                    while (!ok && !*(volatile int *)&abort_flag && global_ns() - t0 <= kWaitLimitNs)
                        ok = mbar_try_wait(empty + 8 * st, ((k / STAGES) - 1) & 1);
                    if (!ok) {
                        atomicExch(a.err, kErrTimeout);
                        abort_flag = 1;
                        break;
                    }
                }
                if (a.inject_skip_plane == k && it == 0) {
                    issued = k;
                    break;
                }
                const bool with_o = k >= 2;
                mbar_arrive_expect_tx(full + 8 * st, S::E_BYTES + (with_o ? S::O_BYTES : 0));
                // padded coordinates: x0-2 -> x0-2+kPadX; E rows from y0-2 -> y0-1, O
                // rows from y0-1 -> y0; plane q = z0-2+k -> z0-1+k
                tma_load_4d(base + st * S::STAGE_BYTES, emap, (w.x0 - 2 + kPadX) * S::XE, w.y0 - 1, 0, w.z0 - 1 + k,
                            full + 8 * st);
                if (with_o)
                    tma_load_4d(base + st * S::STAGE_BYTES + S::O_OFF, omap, (w.x0 - 2 + kPadX) * S::XE, w.y0, 0,
                                w.z0 - 2 + k, full + 8 * st);
                issued = k + 1;
            }
            if (abort_flag) {
                for (int k = (issued > STAGES ? issued - STAGES : 0); k < issued; k++)
                    mbar_wait_bounded(full + 8 * (k % STAGES), (k / STAGES) & 1);
            }
        }
    } else {
        // ---- consumer warps ----------------------------------------------
        const bool in_box = tid < S::EX * S::EY;
        const int ex = in_box ? tid % S::EX : 0, ey = in_box ? tid / S::EX : 0;
        const int x = w.x0 - 1 + ex, y = w.y0 - 1 + ey;
        const bool inside = in_box && x >= 0 && x < d.nx && y >= 0 && y < d.ny;
        const bool tile = inside && ex >= 1 && ex <= TX && ey >= 1 && ey <= TY;
        const long long zstride = d.zstride, plane = d.plane;
        const long long col = inside ? field_index(d, 0, x, y, 0) : 0;
        const long long voff = d.vbase - d.base;
        const T Lw[2] = {T(d.Lc[0]), T(d.Lc[1])};
        const T L0 = T(d.L0), gdt = T(d.gdt);
        T2 *__restrict__ oute = (T2 *)a.out_e;
        T2 *__restrict__ outo = (T2 *)a.out_o;
        const T *__restrict__ vpot = (const T *)a.vpot;
        T vxy0 = T(0), vxy1 = T(0);
        if (POT == GPE_POTENTIAL_TRAP && inside) {
            const T *tx_ = vpot + d.vbase;
            const T *ty_ = tx_ + 2ll * d.nx;
            vxy0 = d_add(tx_[x], ty_[y]);
            vxy1 = d_add(tx_[d.nx + x], ty_[d.ny + y]);
        }
        auto vdt_at = [&](int slot, int z) -> T {  // V*dt at (x, y, z), z in z0-1 .. z1
            if (POT == GPE_POTENTIAL_TRAP) return d_add(slot ? vxy1 : vxy0, ztab[slot * (zl + 2) + z - (w.z0 - 1)]);
            return vpot[col + z * zstride + slot * plane + voff];
        };

        const T2 zero2 = {T(0), T(0)};
        // phase A carries: E at this column (see the one-half-step kernel)
        T2 cm = zero2, cc = zero2, bm = zero2, bc = zero2, axyC = zero2, axyB = zero2, bBp = zero2, sd0 = zero2,
           bCc = zero2;
        // phase B carries: O' at this column
        T2 pcm = zero2, pcc = zero2, pbm = zero2, pbc = zero2, paxyC = zero2, paxyB = zero2, pbBp = zero2,
           psd0 = zero2, pbCc = zero2;
        const int lx = ex + 1, ly = ey + 1;  // E box position of the column
        for (int k = 0; k < nplanes; k++) {
            const int st = k % STAGES;
            // A thread whose wait runs out still reaches the consumers' barrier
            // below, where all of them learn of it and stop together.
            const bool got = mbar_wait_bounded(full + 8 * st, (k / STAGES) & 1);
            if (!got) {
                atomicExch(a.err, kErrTimeout);
                abort_flag = 1;
            }
            const unsigned char *sb = gbase + st * S::STAGE_BYTES;
            const T2 *Ep = (const T2 *)sb;
            const T2 *EB = Ep + S::BW * S::EH;
            auto at = [&](const T2 *P, int dx, int dy) -> T2 { return P[(ly + dy) * S::BW + lx + dx]; };
            const T2 qC = at(Ep, 0, 0), qCxm = at(Ep, -1, 0), qCxp = at(Ep, 1, 0), qCym = at(Ep, 0, -1),
                     qCyp = at(Ep, 0, 1), qCpp = at(Ep, 1, 1);
            const T2 qB = at(EB, 0, 0), qBxm = at(EB, -1, 0), qBxp = at(EB, 1, 0), qBym = at(EB, 0, -1),
                     qByp = at(EB, 0, 1), qBmm = at(EB, -1, -1);
            T2 o0 = zero2, o1 = zero2;  // O(p) at the column, p = q-1
            if (k >= 2) {
                const T2 *Op = (const T2 *)(sb + S::O_OFF);
                o0 = Op[ey * S::BW + lx];
                o1 = Op[S::BW * S::OH + ey * S::BW + lx];
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + 8 * st);

            // ---- phase A: O'(p), p = z0-3+k, from E planes p-1, p, p+1
            const T2 bBq = Ops<T>::add(Ops<T>::add(qBmm, qBym), Ops<T>::add(qBxm, qB));
            const T2 bCq = Ops<T>::add(Ops<T>::add(qC, qCxp), Ops<T>::add(qCyp, qCpp));
            const T2 axyCq = Ops<T>::add(Ops<T>::add(qCxm, qCxp), Ops<T>::add(qCym, qCyp));
            const T2 axyBq = Ops<T>::add(Ops<T>::add(qBxm, qBxp), Ops<T>::add(qBym, qByp));
            const T2 sd0q = Ops<T>::add(bBp, bBq);
            const int p = w.z0 - 3 + k;
            T2 n0 = zero2, n1 = zero2;  // O'(p) of the column; zero outside the instance
            if (k >= 2 && inside && p >= 0 && p < nz) {
                T2 S2[2];
                T hx, hy, nrm;
                S2[0] = sd0;
                S2[1] = Ops<T>::add(Ops<T>::add(cm, qC), axyC);
                Ops<T>::hpsi(cc, S2, Lw, L0, vdt_at(0, p), gdt, hx, hy, nrm);
                n0 = integrate<T, 0>(o0, cc, hx, hy);
                S2[0] = Ops<T>::add(bCc, bCq);
                S2[1] = Ops<T>::add(Ops<T>::add(bm, qB), axyB);
                Ops<T>::hpsi(bc, S2, Lw, L0, vdt_at(1, p), gdt, hx, hy, nrm);
                n1 = integrate<T, 0>(o1, bc, hx, hy);
                if (got && tile && p >= w.z0 && p < w.z1) {
                    const long long i0 = col + p * zstride;
                    outo[i0] = n0;
                    outo[i0 + plane] = n1;
                }
            }
            const T2 eown0 = cm, eown1 = bm;  // E(p-1) of the column, the target of phase B
            cm = cc;
            cc = qC;
            bm = bc;
            bc = qB;
            axyC = axyCq;
            axyB = axyBq;
            bBp = bBq;
            sd0 = sd0q;
            bCc = bCq;

            // ---- hand O'(p) to the tile
            T2 *nb = newbuf + (k & 1) * (S::NEW_BYTES / (int)sizeof(T2));
            if (in_box) {
                nb[ey * S::EX + ex] = n0;
                nb[S::NEW_SLOT + ey * S::EX + ex] = n1;
            }
            if (bar_any(1, NT, !got)) break;  // consumer warps only

            // ---- phase B: E'(p-1) from O' planes p-2, p-1, p (read: plane p)
            if (k >= 2 && ex >= 1 && ex <= TX && ey >= 1 && ey <= TY && in_box) {
                auto nat = [&](int sl, int dx, int dy) -> T2 {
                    return nb[sl * S::NEW_SLOT + (ey + dy) * S::EX + ex + dx];
                };
                const T2 rC = nat(0, 0, 0), rCxm = nat(0, -1, 0), rCxp = nat(0, 1, 0), rCym = nat(0, 0, -1),
                         rCyp = nat(0, 0, 1), rCpp = nat(0, 1, 1);
                const T2 rB = nat(1, 0, 0), rBxm = nat(1, -1, 0), rBxp = nat(1, 1, 0), rBym = nat(1, 0, -1),
                         rByp = nat(1, 0, 1), rBmm = nat(1, -1, -1);
                const T2 pbBq = Ops<T>::add(Ops<T>::add(rBmm, rBym), Ops<T>::add(rBxm, rB));
                const T2 pbCq = Ops<T>::add(Ops<T>::add(rC, rCxp), Ops<T>::add(rCyp, rCpp));
                const T2 paxyCq = Ops<T>::add(Ops<T>::add(rCxm, rCxp), Ops<T>::add(rCym, rCyp));
                const T2 paxyBq = Ops<T>::add(Ops<T>::add(rBxm, rBxp), Ops<T>::add(rBym, rByp));
                const T2 psd0q = Ops<T>::add(pbBp, pbBq);
                const int pz = p - 1;
                if (k >= 4 && inside) {  // pz in z0 .. z1-1
                    T2 S2[2];
                    T hx, hy, nrm;
                    S2[0] = psd0;
                    S2[1] = Ops<T>::add(Ops<T>::add(pcm, rC), paxyC);
                    Ops<T>::hpsi(pcc, S2, Lw, L0, vdt_at(0, pz), gdt, hx, hy, nrm);
                    const T2 e0 = integrate<T, 0>(eown0, pcc, hx, hy);
                    S2[0] = Ops<T>::add(pbCc, pbCq);
                    S2[1] = Ops<T>::add(Ops<T>::add(pbm, rB), paxyB);
                    Ops<T>::hpsi(pbc, S2, Lw, L0, vdt_at(1, pz), gdt, hx, hy, nrm);
                    const T2 e1 = integrate<T, 0>(eown1, pbc, hx, hy);
                    const long long i0 = col + pz * zstride;
                    oute[i0] = e0;
                    oute[i0 + plane] = e1;
                }
                pcm = pcc;
                pcc = rC;
                pbm = pbc;
                pbc = rB;
                paxyC = paxyCq;
                paxyB = paxyBq;
                pbBp = pbBq;
                psd0 = psd0q;
                pbCc = pbCq;
            }
        }
    }
    launch_dependents();
}



// Kernel variants: tile (TX, TY), pipeline depth (STAGES planes) and the
// minimum resident CTAs per SM asked of the register allocator (MINB).  Index 0
// is the default; the autotuner picks among them per workload.
struct Variant {
    int tx, ty, stages, minb;
};
static const Variant kVariants[] = {
    {32, 4, 6, 6}, {32, 4, 4, 6}, {32, 8, 4, 3}, {32, 8, 6, 3}, {32, 4, 8, 5}, {64, 4, 4, 3},
    {16, 8, 6, 6}, {32, 2, 8, 8}, {16, 16, 4, 3}, {32, 8, 4, 2}, {64, 4, 6, 2}, {32, 16, 4, 1},
};

// Variants that advance a whole leapfrog step per launch (twostep_bcc2_kernel):
// output tile (TX, TY), pipeline depth, resident CTAs asked for.  Their indices
// follow the one-half-step variants.
static const Variant kTwoVariants[] = {
    {32, 12, 6, 1}, {32, 4, 4, 2}, {32, 6, 3, 2}, {32, 12, 8, 1}, {32, 8, 3, 1}, {32, 10, 6, 1},
    {32, 10, 3, 1}, {32, 12, 3, 1},
};
constexpr int kOneCount = int(sizeof(kVariants) / sizeof(kVariants[0]));
constexpr int kTwoCount = int(sizeof(kTwoVariants) / sizeof(kTwoVariants[0]));
// The persistent kernel's variants (gpe_persistent.cu) follow the two-step ones.

int fused_tile_count() { return kOneCount + kTwoCount + persistent_variant_count(); }
int fused_variant_kind(int tile)
{
    if (tile >= kOneCount && tile < kOneCount + kTwoCount) return kVariantTwoStep;
    if (tile >= kOneCount + kTwoCount && tile < fused_tile_count()) return kVariantPersistent;
    return kVariantHalfStep;
}
int fused_persistent_index(int tile) { return tile - kOneCount - kTwoCount; }
int fused_half_steps(int tile) { return fused_variant_kind(tile) == kVariantTwoStep ? 2 : 1; }

void fused_variant(int tile, int *tx, int *ty, int *stages, int *minb)
{
    if (tile < 0 || tile >= fused_tile_count()) tile = 0;
    if (fused_variant_kind(tile) == kVariantPersistent) {
        persistent_variant(fused_persistent_index(tile), tx, ty, stages, minb);
        return;
    }
    const Variant &v = tile < kOneCount ? kVariants[tile] : kTwoVariants[tile - kOneCount];
    *tx = v.tx;
    *ty = v.ty;
    *stages = v.stages;
    *minb = v.minb;
}

void fused_tile_shape(int tile, int *tx, int *ty)
{
    int st, mb;
    fused_variant(tile, tx, ty, &st, &mb);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the library
// links only the CUDA runtime); looked up once.
using TensorMapEncode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                     const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static TensorMapEncode tensor_map_encoder()
{
    static TensorMapEncode encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e == cudaSuccess && q == cudaDriverEntryPointSuccess && fn) encode = (TensorMapEncode)fn;
    }
    return encode;
}

// The two 4-D tensor maps of one field of one instance (out_map[0], out_map[1]):
// dimensions (x in 8-byte elements, y, slot, z) over the padded layout; boxes =
// tile plus a 2-column / 1-row halo (previous-field loads) and the interior tile
// (next-field loads), both slots, one plane.  The padded layout puts the
// Dirichlet zeros in memory; boxes that overhang the padded extents are
// zero-filled by the TMA unit.
gpe_status make_halo_map(void *out_map, int precision, const InstDev &d, void *field_arena, int tile)
{
    TensorMapEncode encode = tensor_map_encoder();
    if (!encode) return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    int tx, ty;
    fused_tile_shape(tile, &tx, &ty);
    const int csize = precision == GPE_FP64 ? 16 : 8;
    const int xe = csize / 8;
    const cuuint64_t dims[4] = {(cuuint64_t)d.px * xe, (cuuint64_t)d.py, 2, (cuuint64_t)d.nz + 2};
    const cuuint64_t strides[3] = {(cuuint64_t)d.px * csize, (cuuint64_t)d.plane * csize,
                                   (cuuint64_t)d.zstride * csize};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    void *gaddr = (char *)field_arena + (size_t)d.base * csize;
    // [0]: tile plus halo, both slots, one plane; [1]: interior tile, both slots, one plane
    const cuuint32_t boxes[2][4] = {{(cuuint32_t)(tx + 4) * xe, (cuuint32_t)(ty + 2), 2, 1},
                                    {(cuuint32_t)tx * xe, (cuuint32_t)ty, 2, 1}};
    for (int b = 0; b < 2; b++) {
        CUresult r = encode((CUtensorMap *)out_map + b, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, gaddr, dims, strides,
                            boxes[b], estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    return GPE_OK;
}

gpe_status make_t12_maps(void *out_map, const InstDev &d, void *field_arena, int tx, int ty)
{
    TensorMapEncode encode = tensor_map_encoder();
    if (!encode) return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[4] = {(cuuint64_t)d.px, (cuuint64_t)d.py, (cuuint64_t)d.slots, (cuuint64_t)d.nz + 2};
    const cuuint64_t strides[3] = {(cuuint64_t)d.px * 8, (cuuint64_t)d.plane * 8, (cuuint64_t)d.zstride * 8};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const cuuint32_t boxes[2][4] = {{(cuuint32_t)(tx + 4), (cuuint32_t)(ty + 2), (cuuint32_t)d.slots, 1},
                                    {(cuuint32_t)tx, (cuuint32_t)ty, (cuuint32_t)d.slots, 1}};
    void *gaddr = (char *)field_arena + (size_t)d.base * 8;
    for (int b = 0; b < 2; b++) {
        CUresult r = encode((CUtensorMap *)out_map + b, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, gaddr, dims, strides,
                            boxes[b], estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    return GPE_OK;
}

gpe_status make_t12_vmap(void *out_map, const InstDev &d, void *vbase_arena, int tx, int ty)
{
    TensorMapEncode encode = tensor_map_encoder();
    if (!encode) return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[4] = {(cuuint64_t)d.px, (cuuint64_t)d.py, (cuuint64_t)d.slots, (cuuint64_t)d.nz + 2};
    const cuuint64_t strides[3] = {(cuuint64_t)d.px * 4, (cuuint64_t)d.plane * 4, (cuuint64_t)d.zstride * 4};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const cuuint32_t box[4] = {(cuuint32_t)(tx + 4), (cuuint32_t)ty, (cuuint32_t)d.slots, 1};
    void *gaddr = (char *)vbase_arena + (size_t)d.vbase * 4;
    CUresult r = encode((CUtensorMap *)out_map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, gaddr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GPE_OK;
}

// The residual map of one field of one instance (GPE_FP32C): 4-D over the
// padded layout in 16-bit words (x, y, slot, z; rows of px words, px a multiple
// of 8 so that every row starts on 16 bytes).  The residual of padded column c
// sits at column c - kLoShift, so the map's column X is the instance's column
// x = X and a tile's box is TX columns from x0 (16-byte aligned), TY rows, both
// slots, one plane.
gpe_status make_residual_map(void *out_map, const InstDev &d, void *lo_arena, int tile)
{
    TensorMapEncode encode = tensor_map_encoder();
    if (!encode) return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    int tx, ty;
    fused_tile_shape(tile, &tx, &ty);
    const cuuint64_t dims[4] = {(cuuint64_t)d.px, (cuuint64_t)d.py, 2, (cuuint64_t)d.nz + 2};
    const cuuint64_t strides[3] = {(cuuint64_t)d.px * 2, (cuuint64_t)d.plane * 2, (cuuint64_t)d.zstride * 2};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const cuuint32_t box[4] = {(cuuint32_t)tx, (cuuint32_t)ty, 2, 1};
    void *gaddr = (char *)lo_arena + (size_t)d.base * 2;
    CUresult r = encode((CUtensorMap *)out_map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 4, gaddr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GPE_OK;
}

// The two-step kernel's maps of one buffer set of one instance: out_map[0] the
// E box (tile plus 2 columns either side, 2 rows either side), out_map[1] the O
// box (tile plus 2 columns, 1 row either side); both slots, one plane.
gpe_status make_twostep_maps(void *out_map, int precision, const InstDev &d, void *even_arena, void *odd_arena,
                             int tile)
{
    TensorMapEncode encode = tensor_map_encoder();
    if (!encode) return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    int tx, ty;
    fused_tile_shape(tile, &tx, &ty);
    const int csize = precision == GPE_FP64 ? 16 : 8;
    const int xe = csize / 8;
    const cuuint64_t dims[4] = {(cuuint64_t)d.px * xe, (cuuint64_t)d.py, 2, (cuuint64_t)d.nz + 2};
    const cuuint64_t strides[3] = {(cuuint64_t)d.px * csize, (cuuint64_t)d.plane * csize,
                                   (cuuint64_t)d.zstride * csize};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    void *arenas[2] = {even_arena, odd_arena};
    const cuuint32_t boxes[2][4] = {{(cuuint32_t)(tx + 4) * xe, (cuuint32_t)(ty + 4), 2, 1},
                                    {(cuuint32_t)(tx + 4) * xe, (cuuint32_t)(ty + 2), 2, 1}};
    for (int b = 0; b < 2; b++) {
        void *gaddr = (char *)arenas[b] + (size_t)d.base * csize;
        CUresult r = encode((CUtensorMap *)out_map + b, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, gaddr, dims, strides,
                            boxes[b], estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return fail(GPE_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    return GPE_OK;
}

// FP64 stages are twice as large: half as many (at least 2) fit the same memory.
template <typename T, int ST> struct TwoStages {
    static constexpr int value = sizeof(T) == 8 ? (ST / 2 > 2 ? ST / 2 : 2) : ST;
};

template <typename T, int TX, int TY, int ST0, int MB, int POT>
static cudaError_t launch_two(const TwoStepArgs &a, int grid, cudaStream_t s)
{
    constexpr int ST = TwoStages<T, ST0>::value;
    const int bytes = twostep_smem_bytes<T, TX, TY, ST>(a.zcmax);
    auto kern = twostep_bcc2_kernel<T, TX, TY, POT, ST, MB>;
    static int allowed = 48 * 1024;
    if (bytes > allowed) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        allowed = bytes;
    }
    return launch_pdl(kern, grid, TwoStepShape<T, TX, TY>::NTHREADS, bytes, s, a);
}

template <typename T, int TX, int TY, int ST, int MB>
static cudaError_t launch_two_pot(const FusedLaunch &l, const TwoStepArgs &a, cudaStream_t s)
{
    if (l.potential == GPE_POTENTIAL_ARRAY) return launch_two<T, TX, TY, ST, MB, 0>(a, l.grid, s);
    return launch_two<T, TX, TY, ST, MB, 1>(a, l.grid, s);
}

template <typename T>
static cudaError_t launch_two_tile(const FusedLaunch &l, const TwoStepArgs &a, cudaStream_t s)
{
    switch (l.tile - kOneCount) {  // must list kTwoVariants in order
    case 1: return launch_two_pot<T, 32, 4, 4, 2>(l, a, s);
    case 2: return launch_two_pot<T, 32, 6, 3, 2>(l, a, s);
    case 3: return launch_two_pot<T, 32, 12, 8, 1>(l, a, s);
    case 4: return launch_two_pot<T, 32, 8, 3, 1>(l, a, s);
    case 5: return launch_two_pot<T, 32, 10, 6, 1>(l, a, s);
    case 6: return launch_two_pot<T, 32, 10, 3, 1>(l, a, s);
    case 7: return launch_two_pot<T, 32, 12, 3, 1>(l, a, s);
    default: return launch_two_pot<T, 32, 12, 6, 1>(l, a, s);
    }
}

cudaError_t launch_twostep(const FusedLaunch &l, cudaStream_t s)
{
    TwoStepArgs a;
    a.inst = l.inst;
    a.items = l.items;
    a.maps = (const CUtensorMap *)l.maps;
    a.set = l.src;
    a.zcmax = l.zcmax;
    a.out_e = l.out_e;
    a.out_o = l.out_o;
    a.vpot = l.vpot;
    a.err = l.err;
    a.inject_skip_plane = l.inject_skip_plane;
    if (l.precision == GPE_FP64) return launch_two_tile<double>(l, a, s);
    return launch_two_tile<float>(l, a, s);
}

template <typename T, int TX, int TY, int ST, int MB, int MODE, int POT>
static cudaError_t launch_one(const FusedArgs &a, int grid, cudaStream_t s)
{
    const int bytes = fused_smem_bytes<T, TX, TY, ST, MODE == 2>(a.zcmax);
    auto kern = fused_bcc2_kernel<T, TX, TY, MODE, POT, ST, MB>;
    static int allowed = 48 * 1024;  // dynamic shared memory granted to this instantiation
    if (bytes > allowed) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        allowed = bytes;
    }
    // Real time: programmatic dependent launch.  Imaginary time ends every grid with
    // a serial fold in one CTA; there an early-scheduled next grid only holds SM
    // slots, so it launches plainly (the griddepcontrol instructions are then no-ops).
    if (MODE != 1) return launch_pdl(kern, grid, FusedShape<T, TX, TY>::NTHREADS, bytes, s, a);
    kern<<<grid, FusedShape<T, TX, TY>::NTHREADS, bytes, s>>>(a);
    return cudaGetLastError();
}

template <typename T, int TX, int TY, int ST, int MB>
static cudaError_t fused_launch_t(const FusedLaunch &l, const FusedArgs &a, cudaStream_t s)
{
    if constexpr (sizeof(T) == 4) {
        if (l.mode == GPE_REAL_TIME && l.comp) {
            if (l.potential == GPE_POTENTIAL_ARRAY) return launch_one<T, TX, TY, ST, MB, 2, 0>(a, l.grid, s);
            return launch_one<T, TX, TY, ST, MB, 2, 1>(a, l.grid, s);
        }
    }
    if (l.mode == GPE_REAL_TIME) {
        if (l.potential == GPE_POTENTIAL_ARRAY) return launch_one<T, TX, TY, ST, MB, 0, 0>(a, l.grid, s);
        return launch_one<T, TX, TY, ST, MB, 0, 1>(a, l.grid, s);
    }
    if (l.potential == GPE_POTENTIAL_ARRAY) return launch_one<T, TX, TY, ST, MB, 1, 0>(a, l.grid, s);
    return launch_one<T, TX, TY, ST, MB, 1, 1>(a, l.grid, s);
}

template <typename T>
static cudaError_t fused_launch_tile(const FusedLaunch &l, const FusedArgs &a, cudaStream_t s)
{
    switch (l.tile) {  // must list kVariants in order
    case 1: return fused_launch_t<T, 32, 4, 4, 6>(l, a, s);
    case 2: return fused_launch_t<T, 32, 8, 4, 3>(l, a, s);
    case 3: return fused_launch_t<T, 32, 8, 6, 3>(l, a, s);
    case 4: return fused_launch_t<T, 32, 4, 8, 5>(l, a, s);
    case 5: return fused_launch_t<T, 64, 4, 4, 3>(l, a, s);
    case 6: return fused_launch_t<T, 16, 8, 6, 6>(l, a, s);
    case 7: return fused_launch_t<T, 32, 2, 8, 8>(l, a, s);
    case 8: return fused_launch_t<T, 16, 16, 4, 3>(l, a, s);
    case 9: return fused_launch_t<T, 32, 8, 4, 2>(l, a, s);
    case 10: return fused_launch_t<T, 64, 4, 6, 2>(l, a, s);
    case 11: return fused_launch_t<T, 32, 16, 4, 1>(l, a, s);
    default: return fused_launch_t<T, 32, 4, 6, 6>(l, a, s);
    }
}

cudaError_t launch_fused_step(const FusedLaunch &l, cudaStream_t s)
{
    FusedArgs a;
    a.inst = l.inst;
    a.items = l.items;
    a.num_items = l.num_items;
    a.maps = (const CUtensorMap *)l.maps;
    a.lo_maps = (const CUtensorMap *)l.lo_maps;
    a.zcmax = l.zcmax;
    a.src = l.src;
    a.prev = l.prev;
    a.next = l.next;
    a.next_lo = (uint16_t *)l.next_lo;
    a.vpot = l.vpot;
    a.imag = l.imag;
    a.partials = l.partials;
    a.counter = l.counter;
    a.inst_item_begin = l.inst_item_begin;
    a.num_instances = l.num_instances;
    a.tol = l.tol;
    a.err = l.err;
    a.inject_skip_plane = l.inject_skip_plane;
    if (l.precision == GPE_FP64) return fused_launch_tile<double>(l, a, s);
    return fused_launch_tile<float>(l, a, s);
}

}  // namespace gpe
