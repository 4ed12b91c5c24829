// gpe_persistent.cu - the fused BCC2 real-time half-step as one persistent
// launch that advances every instance of a batch by many half-steps.
//
// The reference drives its leapfrog from the host, two launches per step
// (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:475-481).  Here one
// cooperative launch runs all the half-steps of a gpe_step call.  Its CTAs stay
// resident and take tickets from one counter: ticket t is work item t % N of
// half-step t / N (N items, the same list as the one-launch-per-half-step
// kernel), so every CTA that finishes early takes more work and the CTAs stay
// balanced however unevenly the items divide among them.  Each item runs
// exactly as in that kernel (gpe_fused_core.cuh: the producer lane's TMA issue,
// the consumer warps' z-march), so the results are bit-identical to it.  The
// producer tells its consumers which ticket a ring plane starts with through a
// per-stage tag in shared memory, written before the plane's copies are issued
// and read after its full barrier completes.
//
// Ordering without a grid barrier: item X at half-step h reads the field its
// neighbours wrote at half-step h-1 (halo), and rewrites the field they read
// at h-1, so it may start once every item within one tile / one z-chunk of it
// (at most 27, itself included) has finished h-1.  Each item has an epoch
// word done[X], the half-steps it has completed since the handle was created.
//   * publish: after the item's last plane every consumer thread fences its
//     stores into the async proxy and each consumer warp arrives (CTA scope) on
//     a slot of a small publication ring in shared memory.  A publisher warp
//     waits for all consumer warps of the slot, fences at GPU scope (making
//     their stores visible, by cumulativity) and adds 1 to done[X] with release
//     semantics.  The consumer warps never stall on a GPU-scope fence; they run
//     up to kPub items ahead of the publisher;
//   * wait: before issuing item X at half-step h, lane j of the producer warp
//     polls done[neighbour j] with acquire loads until it reaches epoch0 + h;
//     lane 0 then fences into the async proxy and issues the TMA copies.
// The producer runs ahead of its consumers by the ring's depth across item and
// half-step boundaries, so the pipeline does not drain between half-steps, and
// small and large instances of a batch advance independently.  No CTA waits
// for one that is not resident: the launch is cooperative (the grid is at most
// the resident CTAs).  Nothing deadlocks: tickets are handed out in increasing
// order, a ticket depends only on smaller ones, and each CTA runs its tickets
// in order, so the smallest unfinished ticket always has its dependencies done
// and its CTA working on it.
//
// Waits are bounded (about one second).  A wait that runs out sets the
// handle's error word; every other wait of the launch (epoch polls, ring
// barriers) also watches that word and gives up at once, so a failure ends the
// whole launch promptly.  Each CTA then lets its own copies in flight land and
// returns; the host reports GPE_ERR_TIMEOUT and resets the epoch words.

#include "gpe_fused_core.cuh"

#include <algorithm>

namespace gpe {

struct PersistArgs {
    const InstDev *__restrict__ inst;
    const WorkItem *__restrict__ items;
    int num_items;
    const CUtensorMap *maps;     // [instance][field][halo box, interior box]
    const CUtensorMap *lo_maps;  // MODE 2: [instance][field] residual box
    void *field[2];              // even, odd
    uint16_t *lo[2];             // MODE 2: their int8 x 2 residuals
    const void *vpot;
    unsigned long long *ticket;  // ticket counter, zero at launch
    const int *nbr_begin;        // [num_items + 1]: CSR rows of nbr
    const int *nbr;              // the items each item depends on (itself included)
    unsigned int *done;          // per item: half-steps completed
    unsigned int epoch0;         // half-steps every item had completed when this launch starts
    int half_steps;              // half-steps this launch advances (odd <- even first)
    int *err;
    int inject_skip_plane;       // test hook: plane the producer of item 0 withholds at half-step 0
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_gpu_add(unsigned *p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until *p has reached `need` (epochs compare modulo 2^32); gives up after
// about a second, or as soon as the launch's error word or the CTA's abort flag
// is set.
__device__ __forceinline__ bool wait_epoch(const unsigned *p, unsigned need, const int *gerr,
                                           const volatile int *abort_flag)
{
    if (int(ld_acquire_gpu(p) - need) >= 0) return true;
    const uint64_t t0 = global_ns();
    for (unsigned i = 1;; i++) {
        __nanosleep(64);  // eases the polling load on L2 while CTAs wait for a lagging neighbour
        if (int(ld_acquire_gpu(p) - need) >= 0) return true;
        if ((i & 15u) == 0u && (*(const volatile int *)gerr != 0 || *abort_flag || global_ns() - t0 > kWaitLimitNs))
            return false;
    }
}

constexpr int kPub = 4;  // publication ring slots

// Threads of a persistent CTA: the consumer warps, the producer warp, the publisher warp.
template <typename T, int TX, int TY> constexpr int persistent_threads() { return TX * TY + 64; }

template <typename T, int TX, int TY, int MODE, int POT, int STAGES, int MINB>
__global__ void __launch_bounds__(persistent_threads<T, TX, TY>(), MinBlocks<T, MINB>::value)
    persistent_bcc2_kernel(const PersistArgs a)
{
    static_assert(MODE == 0 || (MODE == 2 && sizeof(T) == 4), "real time: plain or compensated FP32 storage");
    using S = FusedShape<T, TX, TY, MODE == 2>;
    constexpr int NT = S::NT;
    constexpr int NCW = NT / 32;  // consumer warps
    constexpr int PRODUCER = NCW, PUBLISHER = NCW + 1;
    extern __shared__ unsigned char dyn_smem[];
    const uint32_t raw = smem_u32(dyn_smem);
    const uint32_t base = (raw + 127u) & ~127u;
    unsigned char *const gbase = dyn_smem + (base - raw);
    const uint32_t full = base + STAGES * S::STAGE_BYTES;
    const uint32_t empty = full + 8 * STAGES;
    __shared__ volatile int abort_flag;
    __shared__ unsigned long long stage_tag[STAGES];  // ticket whose first plane a stage holds
    __shared__ __align__(8) unsigned long long pub_bar[2 * kPub];  // [slot] full (NCW arrivals), empty (1)
    __shared__ int pub_item[kPub];                                  // item of the slot, -1 = no more
    constexpr unsigned long long kEnd = ~0ull;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        abort_flag = 0;
        for (int st = 0; st < STAGES; st++) {
            mbar_init(full + 8 * st, 1);
            mbar_init(empty + 8 * st, NT / 32);
        }
        for (int j = 0; j < kPub; j++) {
            mbar_init(smem_u32(&pub_bar[2 * j]), NCW);
            mbar_init(smem_u32(&pub_bar[2 * j + 1]), 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const unsigned long long N = (unsigned long long)a.num_items;
    const unsigned long long total = (unsigned long long)a.half_steps * N;

    if (warp == PUBLISHER) {
        // ---- publisher warp: makes each finished item visible at GPU scope --
        if (lane == 0) {
            for (int m = 0;; m++) {
                const int j = m % kPub;
                if (!mbar_wait_watched<true>(smem_u32(&pub_bar[2 * j]), (m / kPub) & 1, a.err)) break;
                const int it = pub_item[j];
                if (it < 0) break;
                __threadfence();  // the consumers' stores, seen through the slot's barrier, come first
                red_release_gpu_add(a.done + it, 1u);
                mbar_arrive(smem_u32(&pub_bar[2 * j + 1]));
            }
        }
    } else if (warp == PRODUCER) {
        // ---- producer warp: tickets and dependency polls on all lanes, TMA issue on lane 0
        int issued = 0;
        bool ended = false;  // the end-of-work plane went out
        while (true) {
            unsigned long long t = 0;
            if (lane == 0) t = atomicAdd(a.ticket, 1ull);
            t = __shfl_sync(0xffffffffu, t, 0);
            const bool aborting = __any_sync(0xffffffffu, abort_flag != 0);  // one decision for the warp
            if (t >= total || aborting) {
                // no more work: an empty plane tagged kEnd tells the consumers
                if (lane == 0 && !aborting) {
                    const int st = issued % STAGES;
                    bool ok = issued < STAGES || mbar_wait_watched<true>(empty + 8 * st, ((issued / STAGES) - 1) & 1,
                                                                         a.err);
                    if (ok) {
                        stage_tag[st] = kEnd;
                        mbar_arrive(full + 8 * st);  // completes the phase with no copies
                        ended = true;
                    }
                }
                break;
            }
            const int h = int(t / N), it = int(t % N);
            const unsigned need = a.epoch0 + unsigned(h);
            const int nb0 = a.nbr_begin[it], nbn = a.nbr_begin[it + 1] - nb0;
            const bool ready = lane >= nbn || wait_epoch(a.done + a.nbr[nb0 + lane], need, a.err, &abort_flag);
            if (__any_sync(0xffffffffu, !ready)) {
                if (lane == 0) {
                    atomicExch(a.err, kErrTimeout);
                    abort_flag = 1;
                }
                break;
            }
            __syncwarp();  // orders the other lanes' acquire loads before lane 0's issue
            int r = kItemDone;
            if (lane == 0) {
                __threadfence();             // the flags the other lanes acquired come first
                fence_proxy_async_global();  // then this CTA's TMA reads of the neighbours' stores
                r = produce_item<T, TX, TY, MODE, STAGES, true>(
                    a.items[it], issued, h & 1, a.maps, a.lo_maps, base, full, empty,
                    (h == 0 && it == 0) ? a.inject_skip_plane : -1, a.err, &abort_flag, issued, stage_tag, t);
            }
            r = __shfl_sync(0xffffffffu, r, 0);
            if (r != kItemDone) break;
        }
        // After an abort, the copies this CTA issued land before it exits.  A
        // normal end needs no wait: the consumers take every plane before the
        // end-of-work plane, and the CTA stays until they finish (the ring's
        // phases have then moved past the ones a drain would test).
        if (lane == 0 && !ended) drain_ring<STAGES>(issued, full);
    } else {
        // ---- consumer warps: finished items go to the publisher ------------
        int kb = 0, m = 0;
        Acc<T> acc[4];
        // slot m of the publication ring takes item `item` (-1: no more); false
        // if the wait for a free slot ran out (the error word is then set)
        auto hand_over = [&](int item) -> bool {
            bool ok = true;
            if (lane == 0) {
                const int j = m % kPub;
                if (m >= kPub) ok = mbar_wait_watched<true>(smem_u32(&pub_bar[2 * j + 1]), ((m / kPub) - 1) & 1, a.err);
                if (ok) {
                    pub_item[j] = item;  // every warp writes the same value
                    mbar_arrive(smem_u32(&pub_bar[2 * j]));
                }
            }
            m++;
            return __shfl_sync(0xffffffffu, ok, 0);
        };
        while (true) {
            // the ticket of the next item, from the tag of its first plane's stage
            const int st = kb % STAGES;
            const bool got = mbar_wait_watched<true>(full + 8 * st, (kb / STAGES) & 1, a.err);
            if (__any_sync(0xffffffffu, !got)) {
                atomicExch(a.err, kErrTimeout);
                abort_flag = 1;
                break;
            }
            const unsigned long long t = stage_tag[st];
            if (t == kEnd) {
                hand_over(-1);
                break;
            }
            const int h = int(t / N), it = int(t % N);
            void *next = (h & 1) ? a.field[0] : a.field[1];  // selects, so the argument arrays stay in registers
            uint16_t *next_lo = (h & 1) ? a.lo[0] : a.lo[1];
            const WorkItem w = a.items[it];
            const InstDev &d = a.inst[w.inst];
            const T *tz = (const T *)a.vpot + d.vbase + 2ll * d.nx + 2ll * d.ny;  // trap: z-terms [slot][z]
            if (!consume_item<T, TX, TY, MODE, POT, STAGES, true>(w, d, kb, gbase, full, empty, next, next_lo,
                                                                  a.vpot, tz, d.nz, 0, T(1), acc, tid, lane, a.err,
                                                                  &abort_flag))
                break;  // warp-uniform; the launch's error word is set, the other warps stop too
            kb += w.z1 - w.z0 + 2;
            fence_proxy_async_global();  // this thread's stores, before other CTAs' TMA reads of them
            __syncwarp();
            if (!hand_over(it)) {
                atomicExch(a.err, kErrTimeout);
                abort_flag = 1;
                break;
            }
        }
    }
}

// Persistent variants: tile (TX, TY), ring depth, resident CTAs asked for; the
// tile shapes are those of the one-launch-per-half-step variants of the same
// name, whose TMA boxes they use.
struct PVariant {
    int tx, ty, stages, minb;
};
static const PVariant kPersistVariants[] = {
    {32, 8, 6, 2}, {32, 4, 8, 4}, {32, 2, 8, 6}, {64, 4, 4, 2}, {32, 16, 4, 1}, {16, 8, 6, 4},
};
constexpr int kPersistCount = int(sizeof(kPersistVariants) / sizeof(kPersistVariants[0]));

int persistent_variant_count() { return kPersistCount; }
void persistent_variant(int k, int *tx, int *ty, int *stages, int *minb)
{
    const PVariant &v = kPersistVariants[(k >= 0 && k < kPersistCount) ? k : 0];
    *tx = v.tx;
    *ty = v.ty;
    *stages = v.stages;
    *minb = v.minb;
}

template <typename T, int TX, int TY, int ST, int MB, int MODE, int POT>
static cudaError_t launch_p(const PersistArgs &a, cudaStream_t s, int device, int *grid_out)
{
    const int bytes = fused_smem_bytes<T, TX, TY, ST, MODE == 2>(0);
    auto kern = persistent_bcc2_kernel<T, TX, TY, MODE, POT, ST, MB>;
    constexpr int threads = persistent_threads<T, TX, TY>();
    static int resident = 0;  // CTAs per SM of this instantiation (the same on every GB300)
    if (resident == 0) {
        if (bytes > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
        }
        int nb = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, bytes);
        if (e != cudaSuccess) return e;
        if (nb < 1) return cudaErrorLaunchOutOfResources;
        resident = nb;
    }
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    const int grid = std::min(a.num_items, resident * sms);
    *grid_out = grid;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident at once
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(unsigned(threads));
    cfg.dynamicSmemBytes = size_t(bytes);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

template <typename T, int TX, int TY, int ST, int MB>
static cudaError_t launch_p_mode(const PersistLaunch &l, const PersistArgs &a, cudaStream_t s, int *grid)
{
    if constexpr (sizeof(T) == 4) {
        if (l.comp) {
            if (l.potential == GPE_POTENTIAL_ARRAY) return launch_p<T, TX, TY, ST, MB, 2, 0>(a, s, l.device, grid);
            return launch_p<T, TX, TY, ST, MB, 2, 1>(a, s, l.device, grid);
        }
    }
    if (l.potential == GPE_POTENTIAL_ARRAY) return launch_p<T, TX, TY, ST, MB, 0, 0>(a, s, l.device, grid);
    return launch_p<T, TX, TY, ST, MB, 0, 1>(a, s, l.device, grid);
}

template <typename T>
static cudaError_t launch_p_variant(const PersistLaunch &l, const PersistArgs &a, cudaStream_t s, int *grid)
{
    switch (l.variant) {  // must list kPersistVariants in order
    case 1: return launch_p_mode<T, 32, 4, 8, 4>(l, a, s, grid);
    case 2: return launch_p_mode<T, 32, 2, 8, 6>(l, a, s, grid);
    case 3: return launch_p_mode<T, 64, 4, 4, 2>(l, a, s, grid);
    case 4: return launch_p_mode<T, 32, 16, 4, 1>(l, a, s, grid);
    case 5: return launch_p_mode<T, 16, 8, 6, 4>(l, a, s, grid);
    default: return launch_p_mode<T, 32, 8, 6, 2>(l, a, s, grid);
    }
}

cudaError_t launch_persistent(const PersistLaunch &l, cudaStream_t s, int *grid)
{
    PersistArgs a;
    a.inst = l.inst;
    a.items = l.items;
    a.num_items = l.num_items;
    a.maps = (const CUtensorMap *)l.maps;
    a.lo_maps = (const CUtensorMap *)l.lo_maps;
    a.field[0] = l.field[0];
    a.field[1] = l.field[1];
    a.lo[0] = (uint16_t *)l.lo[0];
    a.lo[1] = (uint16_t *)l.lo[1];
    a.vpot = l.vpot;
    a.ticket = l.ticket;
    a.nbr_begin = l.nbr_begin;
    a.nbr = l.nbr;
    a.done = l.done;
    a.epoch0 = l.epoch0;
    a.half_steps = l.half_steps;
    a.err = l.err;
    a.inject_skip_plane = l.inject_skip_plane;
    if (l.precision == GPE_FP64) return launch_p_variant<double>(l, a, s, grid);
    return launch_p_variant<float>(l, a, s, grid);
}

}  // namespace gpe
