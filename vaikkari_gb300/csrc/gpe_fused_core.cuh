// gpe_fused_core.cuh - device code shared by the fused BCC2 half-step kernel
// (gpe_fused.cu, one launch per half-step) and the persistent kernel
// (gpe_persistent.cu, one launch for many half-steps): PTX helpers for the
// mbarrier/TMA pipeline, packed FP32 pair arithmetic, and the two halves of one
// work item's pass - the producer lane's TMA issue of its planes and the
// consumer threads' z-march (stencil, potential, nonlinearity, update).
//
// Ring numbering: the planes of all items a CTA processes in one launch form
// one sequence through its STAGES-deep shared-memory ring.  Plane number n
// (counted over every item the CTA has run so far in the launch) uses stage
// n % STAGES and phase (n / STAGES) & 1 of that stage's "full" and "empty"
// mbarriers; an item starts at n = kb, its planes before it.  The one-launch-
// per-half-step kernel runs one item per CTA (kb = 0).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>

#include "gpe_internal.h"

namespace gpe {

template <typename T> struct Acc;
template <> struct Acc<double> {
    double s = 0.0;
    __device__ void add(double v) { s += v; }
    __device__ double value() const { return s; }
};
template <> struct Acc<float> {  // compensated FP32
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

// ---- PTX helpers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after about one second of wall time.
constexpr uint64_t kWaitLimitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitLimitNs) return false;
    }
}

// The same, also giving up as soon as the launch's error word is set (WATCH:
// the persistent kernel, where one CTA's timeout must stop every other CTA's
// waits without each running out its own second).
template <bool WATCH>
__device__ __forceinline__ bool mbar_wait_watched(uint32_t bar, uint32_t parity, const int *gerr)
{
    if (!WATCH) return mbar_wait_bounded(bar, parity);
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (unsigned i = 1;; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63u) == 0u && (*(const volatile int *)gerr != 0 || global_ns() - t0 > kWaitLimitNs)) return false;
    }
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

constexpr int kErrTimeout = 1;

template <typename T, int TX, int TY, bool COMP = false>
struct FusedShape {
    using T2 = typename Cplx<T>::type;
    static constexpr int NT = TX * TY;       // consumer threads
    static constexpr int NTHREADS = NT + 32; // plus the producer warp
    static constexpr int BW = TX + 4;        // x0-2 .. x0+TX+1
    static constexpr int BH = TY + 2;        // y0-1 .. y0+TY
    static constexpr int SLOT = BW * BH;
    static constexpr int HALO_BYTES = 2 * SLOT * (int)sizeof(T2);
    static constexpr int NEXT_BYTES = 2 * TX * TY * (int)sizeof(T2);
    static constexpr int NEXT_OFF = ((HALO_BYTES + 127) / 128) * 128;
    // compensated storage: the residual tile (16 bits per value), columns
    // x0 .. x0+TX-1, TY rows, both slots (residuals sit kLoShift places before
    // their values, so the tile's box starts on its first column)
    static constexpr int LO_W = TX;
    static constexpr int LO_BYTES = COMP ? 2 * TY * LO_W * 2 : 0;
    static constexpr int LO_OFF = ((NEXT_OFF + NEXT_BYTES + 127) / 128) * 128;
    static constexpr int STAGE_BYTES = ((LO_OFF + LO_BYTES + 127) / 128) * 128;
    static constexpr int XE = (int)sizeof(T2) / 8;  // 8-byte TMA elements per complex
};

template <typename T, int TX, int TY, int STAGES, bool COMP = false>
int fused_smem_bytes(int zcmax)
{
    return STAGES * FusedShape<T, TX, TY, COMP>::STAGE_BYTES + 128 /* align */ + 16 * STAGES /* barriers */ +
           2 * zcmax * (int)sizeof(T) + 16;
}

// FP64 values need twice the registers: ask for half the resident CTAs.
template <typename T, int MINB> struct MinBlocks {
    static constexpr int value = sizeof(T) == 8 ? (MINB + 1) / 2 : MINB;
};

// Programmatic dependent launch (sm_90 and later).
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch with programmatic stream serialisation: the kernel may begin while the
// previous kernel on the stream drains, and waits for it in grid_dependency_wait.
template <typename Kern, typename Args>
static cudaError_t launch_pdl(Kern kern, int grid, int threads, int bytes, cudaStream_t s, const Args &a)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(unsigned(threads));
    cfg.dynamicSmemBytes = size_t(bytes);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// Complex sums and dt*H psi (gpe_device.cuh's hpsi, two classes) with the same
// rounded operations, packed for FP32.
template <typename T> struct Ops;
template <> struct Ops<double> {
    static __device__ __forceinline__ double2 add(double2 a, double2 b) { return c_add<double>(a, b); }
    static __device__ __forceinline__ void hpsi(double2 p, const double2 *S, const double *L, double L0, double vdt,
                                                double gdt, double &hx, double &hy, double &nrm)
    {
        gpe::hpsi<double, 2>(p, S, L, L0, vdt, gdt, hx, hy, nrm);
    }
};
template <> struct Ops<float> {
    static __device__ __forceinline__ float2 add(float2 a, float2 b) { return f2_add(a, b); }
    static __device__ __forceinline__ void hpsi(float2 p, const float2 *S, const float *L, float L0, float vdt,
                                                float gdt, float &hx, float &hy, float &nrm)
    {
        nrm = d_fma(p.x, p.x, d_mul(p.y, p.y));
        const float c = d_fma(gdt, nrm, d_add(L0, vdt));
        float2 a = f2_mul(make_float2(L[0], L[0]), S[0]);
        a = f2_fma(make_float2(L[1], L[1]), S[1], a);
        const float2 h = f2_fma(make_float2(c, c), p, a);
        hx = h.x;
        hy = h.y;
    }
};

// Compensated update of one value (MODE 2): returns the new stored value and
// replaces lo (int8 residuals of x and y in its low 16 bits, units of the
// stored value's ulp / 256, gpe_device.cuh) with the new residual.
__device__ __forceinline__ float2 integrate_comp(float2 n, float hx, float hy, uint32_t &lo)
{
    const float2 t = f2_add(make_float2(comp_decode(lo, n.x), comp_decode(lo >> 8, n.y)), make_float2(hy, -hx));
    const float2 s = f2_add(n, t);
    const float2 b = f2_sub(s, n);
    const float2 r = f2_add(f2_sub(n, f2_sub(s, b)), f2_sub(t, b));
    lo = comp_encode(r.x, s.x) | (comp_encode(r.y, s.y) << 8);
    return s;
}

// Barrier of threads 0..n-1 on barrier id, returning whether any of them passed v.
__device__ __forceinline__ bool bar_any(int id, int n, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred q, p;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %2, %3, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}



// Cross-proxy fence: orders this thread's generic-proxy global accesses with
// async-proxy (TMA) accesses to global memory.
__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// ---- One work item: producer side ------------------------------------------
// Issues the item's planes q = z0-1 .. z1 into the ring (one lane): the
// previous field's halo box of plane q and, in real time from the third plane
// on, the next field's interior box of plane q-1 (and in MODE 2 its residual
// box), all signalled on the stage's full barrier.  Before reusing a stage it
// waits (bounded) for the empty barrier of the plane STAGES earlier.
// Returns kItemDone, kItemWithheld (test hook: plane `withhold` of this item
// was not issued, nor anything after it) or kItemAbort (a wait ran out or the
// CTA is stopping; *err and *abort_flag are set).  `issued` is the ring number
// one past the last plane issued.  With a non-null `tag`, tag[stage] = tag_value
// is written for the item's first plane once that stage is free, before its
// copies are issued (the persistent kernel names the item to its consumers so).
constexpr int kItemDone = 0, kItemWithheld = 1, kItemAbort = -1;

template <typename T, int TX, int TY, int MODE, int STAGES, bool WATCH>
__device__ __forceinline__ int produce_item(const WorkItem &w, int kb, int src, const CUtensorMap *maps,
                                            const CUtensorMap *lo_maps, uint32_t base, uint32_t full, uint32_t empty,
                                            int withhold, int *err, volatile int *abort_flag, int &issued,
                                            volatile unsigned long long *tag = nullptr,
                                            unsigned long long tag_value = 0)
{
    using S = FusedShape<T, TX, TY, MODE == 2>;
    constexpr bool REAL = MODE != 1;
    const CUtensorMap *halo = maps + 4 * w.inst + 2 * src;
    const CUtensorMap *inner = maps + 4 * w.inst + 2 * (1 - src) + 1;
    const int nplanes = w.z1 - w.z0 + 2;
    for (int k = 0; k < nplanes; k++) {
        const int n = kb + k;
        const int st = n % STAGES;
        if (n >= STAGES) {
            const uint32_t par = ((n / STAGES) - 1) & 1;
            bool ok = mbar_try_wait(empty + 8 * st, par);
            const uint64_t t0 = global_ns();
            for (unsigned i = 1; !ok; i++) {
                if (*abort_flag || global_ns() - t0 > kWaitLimitNs) break;
                if (WATCH && (i & 63u) == 0u && *(const volatile int *)err != 0) break;
                ok = mbar_try_wait(empty + 8 * st, par);
            }
            if (!ok) {
                atomicExch(err, kErrTimeout);
                *abort_flag = 1;
                return kItemAbort;
            }
        }
        if (withhold == k) return kItemWithheld;
        if (k == 0 && tag) tag[st] = tag_value;
        const bool with_next = REAL && (k >= 2);
        mbar_arrive_expect_tx(full + 8 * st, S::HALO_BYTES + (with_next ? S::NEXT_BYTES + S::LO_BYTES : 0));
        // padded coordinates: x0-2 -> x0-2+kPadX, y0-1 -> y0, plane q -> q+1
        tma_load_4d(base + st * S::STAGE_BYTES, halo, (w.x0 - 2 + kPadX) * S::XE, w.y0, 0, w.z0 + k, full + 8 * st);
        if (with_next)  // next field, interior tile of plane q-1 = z0+k-2
            tma_load_4d(base + st * S::STAGE_BYTES + S::NEXT_OFF, inner, (w.x0 + kPadX) * S::XE, w.y0 + 1, 0,
                        w.z0 + k - 1, full + 8 * st);
        if (MODE == 2 && with_next)  // its residuals (columns x0.. in the residual rows)
            tma_load_4d(base + st * S::STAGE_BYTES + S::LO_OFF, lo_maps + 2 * w.inst + (1 - src), w.x0, w.y0 + 1, 0,
                        w.z0 + k - 1, full + 8 * st);
        issued = n + 1;
    }
    return kItemDone;
}

// Lets the copies of the last STAGES planes issued land (bounded) before the
// CTA exits after an abort.
template <int STAGES>
__device__ __forceinline__ void drain_ring(int issued, uint32_t full)
{
    for (int n = (issued > STAGES ? issued - STAGES : 0); n < issued; n++)
        mbar_wait_bounded(full + 8 * (n % STAGES), (n / STAGES) & 1);
}

// ---- One work item: consumer side -------------------------------------------
// Thread tid < TX*TY owns block column (x0 + tid % TX, y0 + tid / TX) of the
// item and marches its planes: reads each plane's stencil from the ring once,
// releases the stage (one arrival per warp), carries what later planes need in
// registers (see the summation order in gpe_fused.cu), and stores the updated
// next field (and in MODE 2 its residuals) with coalesced row writes.  The
// trap potential's z-term of plane z is zt[zt_base_offset(slot) + z - zt_base]
// (shared memory in the one-launch kernel, the instance's table in global
// memory in the persistent one).  MODE 1 (imaginary time) scales the previous
// field by sig as it is read and adds the four sums into acc.  A wait that runs
// out (on any lane of a warp) sets *err and *abort_flag and returns false for
// the whole warp.
template <typename T, int TX, int TY, int MODE, int POT, int STAGES, bool WATCH>
__device__ __forceinline__ bool consume_item(const WorkItem &w, const InstDev &d, int kb, const unsigned char *gbase,
                                             uint32_t full, uint32_t empty, void *next, uint16_t *next_lo,
                                             const void *vpot_, const T *zt, int zt_stride, int zt_base, T sig,
                                             Acc<T> (&acc)[4], int tid, int lane, int *err, volatile int *abort_flag)
{
    using S = FusedShape<T, TX, TY, MODE == 2>;
    using T2 = typename S::T2;
    constexpr bool REAL = MODE != 1;
    const int nplanes = w.z1 - w.z0 + 2;
    const int tx = tid % TX, ty = tid / TX;
    const int x = w.x0 + tx, y = w.y0 + ty;
    const bool valid = (x < d.nx) && (y < d.ny);
    const long long zstride = d.zstride, plane = d.plane;
    const long long col = field_index(d, 0, x, y, 0);
    const long long voff = d.vbase - d.base;
    const T Lw[2] = {T(d.Lc[0]), T(d.Lc[1])};
    const T L0 = T(d.L0), gdt = T(d.gdt);
    T2 *__restrict__ nxt = (T2 *)next;
    uint16_t *__restrict__ nlo = next_lo;
    uint32_t lo0 = 0u, lo1 = 0u;  // MODE 2: residuals of the output plane
    const T *__restrict__ vpot = (const T *)vpot_;
    T vxy0 = T(0), vxy1 = T(0);
    if (POT == GPE_POTENTIAL_TRAP && valid) {
        const T *tx_ = vpot + d.vbase;
        const T *ty_ = tx_ + 2ll * d.nx;
        vxy0 = d_add(tx_[x], ty_[y]);
        vxy1 = d_add(tx_[d.nx + x], ty_[d.ny + y]);
    }

    // carried state (see the summation order in gpe_fused.cu)
    const T2 zero2 = {T(0), T(0)};
    T2 cm = zero2, cc = zero2, bm = zero2, bc = zero2;  // own C, B at planes z-1, z
    T2 axyC = zero2, axyB = zero2;                        // in-plane axial sums at plane z
    T2 bBp = zero2, sd0 = zero2, bCc = zero2;             // bB(z), Sd of slot 0 at z, bC(z)
    const int lx = tx + 2, ly = ty + 1;
    for (int k = 0; k < nplanes; k++) {
        const int n = kb + k;
        const int st = n % STAGES;
        const bool got = mbar_wait_watched<WATCH>(full + 8 * st, (n / STAGES) & 1, err);
        if (__any_sync(0xffffffffu, !got)) {
            atomicExch(err, kErrTimeout);
            *abort_flag = 1;
            return false;
        }
        const unsigned char *sb = gbase + st * S::STAGE_BYTES;
        const T2 *Cp = (const T2 *)sb;
        const T2 *Bp = Cp + S::SLOT;
        auto at = [&](const T2 *P, int dx, int dy) -> T2 {
            T2 v = P[(ly + dy) * S::BW + lx + dx];
            if (MODE == 1) v = c_scale<T>(sig, v);
            return v;
        };
        const T2 qC = at(Cp, 0, 0), qCxm = at(Cp, -1, 0), qCxp = at(Cp, 1, 0), qCym = at(Cp, 0, -1),
                 qCyp = at(Cp, 0, 1), qCpp = at(Cp, 1, 1);
        const T2 qB = at(Bp, 0, 0), qBxm = at(Bp, -1, 0), qBxp = at(Bp, 1, 0), qBym = at(Bp, 0, -1),
                 qByp = at(Bp, 0, 1), qBmm = at(Bp, -1, -1);
        T2 n0 = zero2, n1 = zero2;
        if (REAL && k >= 2) {
            const T2 *Np = (const T2 *)(sb + S::NEXT_OFF);
            n0 = Np[ty * TX + tx];
            n1 = Np[TX * TY + ty * TX + tx];
            if (MODE == 2) {
                const uint16_t *Lp = (const uint16_t *)(sb + S::LO_OFF);
                lo0 = Lp[ty * S::LO_W + tx];
                lo1 = Lp[(TY + ty) * S::LO_W + tx];
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + 8 * st);  // this warp is done with stage st

        // sums of plane q = z0-1+k
        const T2 bBq = Ops<T>::add(Ops<T>::add(qBmm, qBym), Ops<T>::add(qBxm, qB));
        const T2 bCq = Ops<T>::add(Ops<T>::add(qC, qCxp), Ops<T>::add(qCyp, qCpp));
        const T2 axyCq = Ops<T>::add(Ops<T>::add(qCxm, qCxp), Ops<T>::add(qCym, qCyp));
        const T2 axyBq = Ops<T>::add(Ops<T>::add(qBxm, qBxp), Ops<T>::add(qBym, qByp));
        const T2 sd0q = Ops<T>::add(bBp, bBq);  // Sd of slot 0 at plane q

        if (k >= 2 && valid) {
            const int z = w.z0 + k - 2;  // output plane (q - 1)
            T2 S2[2];
            T hx, hy, nrm;
            T v0, v1;
            if (POT == GPE_POTENTIAL_TRAP) {
                v0 = d_add(vxy0, zt[z - zt_base]);
                v1 = d_add(vxy1, zt[zt_stride + z - zt_base]);
            } else {
                const long long i0 = col + z * zstride;
                v0 = vpot[i0 + voff];
                v1 = vpot[i0 + plane + voff];
            }
            // slot 0 (cube corner)
            S2[0] = sd0;
            S2[1] = Ops<T>::add(Ops<T>::add(cm, qC), axyC);
            Ops<T>::hpsi(cc, S2, Lw, L0, v0, gdt, hx, hy, nrm);
            T2 o0;
            if constexpr (MODE == 2) o0 = integrate_comp(n0, hx, hy, lo0);
            else o0 = integrate<T, MODE>(n0, cc, hx, hy);
            if (MODE == 1) {
                acc[0].add(nrm);
                acc[1].add(d_fma(cc.x, hx, d_mul(cc.y, hy)));
                acc[2].add(d_mul(nrm, nrm));
                acc[3].add(d_fma(o0.x, o0.x, d_mul(o0.y, o0.y)));
            }
            // slot 1 (cube centre)
            S2[0] = Ops<T>::add(bCc, bCq);
            S2[1] = Ops<T>::add(Ops<T>::add(bm, qB), axyB);
            Ops<T>::hpsi(bc, S2, Lw, L0, v1, gdt, hx, hy, nrm);
            T2 o1;
            if constexpr (MODE == 2) o1 = integrate_comp(n1, hx, hy, lo1);
            else o1 = integrate<T, MODE>(n1, bc, hx, hy);
            if (MODE == 1) {
                acc[0].add(nrm);
                acc[1].add(d_fma(bc.x, hx, d_mul(bc.y, hy)));
                acc[2].add(d_mul(nrm, nrm));
                acc[3].add(d_fma(o1.x, o1.x, d_mul(o1.y, o1.y)));
            }
            const long long i0 = col + z * zstride;
            nxt[i0] = o0;
            nxt[i0 + plane] = o1;
            if (MODE == 2) {
                nlo[i0 - kLoShift] = uint16_t(lo0);
                nlo[i0 + plane - kLoShift] = uint16_t(lo1);
            }
        }
        cm = cc;
        cc = qC;
        bm = bc;
        bc = qB;
        axyC = axyCq;
        axyB = axyBq;
        bBp = bBq;
        sd0 = sd0q;
        bCc = bCq;
    }
    return true;
}

// ---- Imaginary time: the end of a work item ----------------------------------
// Every thread of the CTA calls this after the item's four sums are in
// row_sums: the first lane of warp pub_warp (a warp with no field stores in
// flight, so its fence waits only for the row) publishes the row; the last CTA
// to finish folds every instance's rows and updates its scalars.
template <int NWARPS>
__device__ __forceinline__ void imag_publish_and_fold(int it, const double *row_sums, volatile int &abort_flag,
                                                      int pub_warp, double *partials, unsigned int *counter,
                                                      const int *inst_item_begin, int num_instances,
                                                      const InstDev *inst, ImagScalars *imag, double tol)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // Last CTA to finish reduces every instance's rows (fixed order).  (A fence
    // in a consumer thread would wait for all of that thread's output stores.)
    __shared__ bool last;
    __syncthreads();
    if (abort_flag) return;
    if (warp == pub_warp && lane == 0) {
        for (int k = 0; k < 4; k++) partials[4ll * it + k] = row_sums[k];
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
        if (last) __threadfence();
    }
    __syncthreads();
    if (!last) return;
    // Each instance's rows are folded by one warp, the instances taken
    // round-robin by the warps, so a batch folds its instances in parallel.
    // Lane l takes rows b+l, b+l+32, ... in groups of eight: the group is
    // added as a fixed pairwise tree (short FP64 dependency chains), the
    // group sums are accumulated in order with compensation, then a fixed
    // xor tree combines the lanes.  The order depends only on the
    // instance's own rows, so an instance gives the same result alone or in
    // any batch.
    for (int i = warp; i < num_instances; i += NWARPS) {
        const int b = inst_item_begin[2 * i], e = inst_item_begin[2 * i + 1];
        double sk[4] = {0.0, 0.0, 0.0, 0.0}, ck[4] = {0.0, 0.0, 0.0, 0.0};
        for (int r0 = b; r0 < e; r0 += 8 * 32) {
            double v[8][4];
#pragma unroll
            for (int u = 0; u < 8; u++) {  // the loads first; rows past the end add zero
                const int r = r0 + u * 32 + lane;
                double2 v01 = make_double2(0.0, 0.0), v23 = make_double2(0.0, 0.0);
                if (r < e) {
                    v01 = __ldcg((const double2 *)(partials + 4ll * r));
                    v23 = __ldcg((const double2 *)(partials + 4ll * r + 2));
                }
                v[u][0] = v01.x;
                v[u][1] = v01.y;
                v[u][2] = v23.x;
                v[u][3] = v23.y;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const double g8 = ((v[0][k] + v[1][k]) + (v[2][k] + v[3][k])) +
                                  ((v[4][k] + v[5][k]) + (v[6][k] + v[7][k]));
                const double yv = g8 - ck[k];
                const double t = sk[k] + yv;
                ck[k] = (t - sk[k]) - yv;
                sk[k] = t;
            }
        }
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) sk[k] += __shfl_xor_sync(0xffffffffu, sk[k], off);
        }
        // sk (every lane): |p'|^2, Re(conj(p') dt H p'), |p'|^4, |next|^2 over values.
        // Lanes 0, 1, 2 form mu, the energy's t1/dt and sigma with one
        // division in lockstep (FP64 division is long-latency here).
        const InstDev &di = inst[i];
        ImagScalars &sc = imag[i];
        const double sq = sqrt(di.vol * sk[3]);
        const double num = (lane == 2) ? 1.0 : sk[1];
        const double den = (lane == 0) ? di.dt * sk[0] : (lane == 1) ? di.dt : sq;
        const double q = num / den;
        if (lane == 0) {
            const double mu = q;
            sc.mu_prev = sc.mu;
            sc.mu = mu;
            sc.dmu = (sc.steps > 0) ? fabs(mu - sc.mu_prev) : INFINITY;
            if (sc.steps > 0 && sc.conv_step < 0 && sc.dmu < tol) sc.conv_step = sc.steps;
            sc.steps += 1;
        } else if (lane == 1) {
            sc.norm_in = di.vol * sk[0];
            sc.energy = di.vol * (q - 0.5 * di.g * sk[2]);
        } else if (lane == 2) {
            sc.sigma = q;
        }
    }
    if (tid == 0) *counter = 0u;
}

}  // namespace gpe
