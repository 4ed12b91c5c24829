// gpe_setup.cu - the per-value part of integrateInTime's set-up on the GPU.
//
// integrateInTime (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:245-348)
// samples, for each of the 12 values of every block, its circumcentre position,
// psi from the vortex profile (VortexState::getPsi, VortexState.cpp:204-238) and
// potentialV3 (GPUGrossPitaevskii_BCC.cu:33-36), and takes the maximum of
// V + g|psi|^2 for the time step.  It then multiplies psi by (1 + noise) drawn
// from the MT19937 stream and forms the odd field with the half-step phase.
//
// Here one thread handles one value.  Every expression is written with the
// correctly rounded FP64 intrinsics (__dadd_rn, __dsub_rn, __dmul_rn, __ddiv_rn,
// __dsqrt_rn), which the compiler never contracts into fused multiply-adds, in
// the reference's operation order.  Each value therefore equals the host
// restatement (compiled with -ffp-contract=off) bit for bit.  The maximum is
// exact in any order: the non-negative candidates are compared as 64-bit
// integers, whose order is the order of their values.
//
// The noise stream stays on the host: getUniformCircle rejects pairs, so which
// draws belong to which value is known only by running the stream in order.
// The host passes each value's accepted pair as the two int32 that the
// reference scales by 2^-31; the scaling is exact, so it is redone here.

#include <cuda_runtime.h>

#include <cstdint>

#include "gpe_internal.h"

namespace gpe {
namespace {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }

// VortexState::getFunction (VortexState.cpp:220-238): bilinear f(r, |z|), zero
// outside the table.  `rr < rsize` is tested before the conversion to an index,
// which equals the host's test after it for every r the conversion can hold.
__device__ double vortex_function(const SetupGeometry &geo, const double *__restrict__ f, double r, double z)
{
    const double rr = __ddiv_rn(sub(r, geo.rplug), geo.rstep);
    if (rr < 0.0) return 0.0;
    if (!(rr < double(geo.rsize))) return 0.0;
    const uint32_t ir = uint32_t(rr);
    const double dr = sub(rr, double(ir));
    const double zz = __ddiv_rn(fabs(z), geo.zstep);
    if (!(zz < double(geo.zsize))) return 0.0;
    const uint32_t iz = uint32_t(zz);
    const double dz = sub(zz, double(iz));
    const size_t ii = size_t(ir) * geo.zsize + iz;
    const bool rn = ir + 1 < geo.rsize, zn = iz + 1 < geo.zsize;
    const double f00 = f[ii];
    const double fr = rn ? f[ii + geo.zsize] : 0.0;
    const double fz = zn ? f[ii + 1] : 0.0;
    const double frz = rn && zn ? f[ii + geo.zsize + 1] : 0.0;
    const double odr = sub(1.0, dr);
    const double a = add(mul(odr, f00), mul(dr, fr));
    const double b = add(mul(odr, fz), mul(dr, frz));
    return add(mul(sub(1.0, dz), a), mul(dz, b));
}

__global__ void __launch_bounds__(256) setup_sample_kernel(SetupGeometry geo, const double *__restrict__ f,
                                                           double2 *__restrict__ psi0, double *__restrict__ V,
                                                           unsigned long long *__restrict__ maxbits,
                                                           unsigned long long nvals)
{
    double m = 0.0;
    for (unsigned long long ii = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; ii < nvals;
         ii += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t l = uint32_t(ii % 12);
        unsigned long long b = ii / 12;
        const uint32_t i = uint32_t(b % geo.nx);
        b /= geo.nx;
        const uint32_t j = uint32_t(b % geo.ny);
        const uint32_t kz = uint32_t(b / geo.ny);
        // p0 + bs * (index * BLOCK_WIDTH + circumcentre offset), per axis
        const double px = add(geo.p0[0], mul(geo.bs, add(mul(double(i), geo.W), geo.bpos[l][0])));
        const double py = add(geo.p0[1], mul(geo.bs, add(mul(double(j), geo.W), geo.bpos[l][1])));
        const double pz = add(geo.p0[2], mul(geo.bs, add(mul(double(kz), geo.W), geo.bpos[l][2])));
        const double rxy = add(mul(px, px), mul(py, py));
        // getPsi: f(r, z) * ((x + i y) / r)^kappa by repeated multiplication
        double cr = 0.0, ci = 0.0;
        const double r = __dsqrt_rn(rxy);
        if (!(r < 1e-30)) {
            cr = vortex_function(geo, f, r, pz);
            const double nr = __ddiv_rn(px, r), ni = __ddiv_rn(py, r);
            for (uint32_t k = 0; k < geo.kappa; k++) {
                const double t = cr;
                cr = sub(mul(t, nr), mul(ci, ni));
                ci = add(mul(ci, nr), mul(t, ni));
            }
        }
        psi0[ii] = make_double2(cr, ci);
        // potentialV3: 0.5 * (x^2 + y^2 + RATIO^2 z^2)
        const double v = mul(0.5, add(rxy, mul(mul(mul(geo.ratio, geo.ratio), pz), pz)));
        V[ii] = v;
        const double poti = add(v, mul(geo.coupling, add(mul(cr, cr), mul(ci, ci))));
        if (poti > m) m = poti;
    }
    // m >= 0 and never NaN: a plain maximum over the warp, then one atomic
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

__device__ __forceinline__ void put(double2 *p, double x, double y) { *p = make_double2(x, y); }
__device__ __forceinline__ void put(float2 *p, double x, double y)
{
    *p = make_float2(__double2float_rn(x), __double2float_rn(y));
}
__device__ __forceinline__ void put(double *p, double x) { *p = x; }
__device__ __forceinline__ void put(float *p, double x) { *p = __double2float_rn(x); }

// psi * (1 + noise) for the even field, times getPhase(-dt/2) for the odd one
// (GPUGrossPitaevskii_BCC.cu:325-348); V copied in the output's element type.
template <typename T>
__global__ void __launch_bounds__(256) setup_noise_kernel(const double2 *__restrict__ psi0,
                                                          const int2 *__restrict__ noise,
                                                          const double *__restrict__ V, double amplitude,
                                                          double ph0, double ph1,
                                                          typename Vec2<T>::type *__restrict__ even,
                                                          typename Vec2<T>::type *__restrict__ odd,
                                                          T *__restrict__ pot, unsigned long long nvals)
{
    const double s = 1.0 / 2147483648.0;
    for (unsigned long long ii = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; ii < nvals;
         ii += (unsigned long long)gridDim.x * blockDim.x) {
        const int2 q = noise[ii];
        const double cx = mul(amplitude, mul(s, double(q.x)));
        const double cy = mul(amplitude, mul(s, double(q.y)));
        const double nr = add(cx, 1.0), ni = cy;
        const double2 p = psi0[ii];
        const double er = sub(mul(p.x, nr), mul(p.y, ni));
        const double ei = add(mul(p.y, nr), mul(p.x, ni));
        put(even + ii, er, ei);
        put(odd + ii, sub(mul(ph0, er), mul(ph1, ei)), add(mul(ph1, er), mul(ph0, ei)));
        put(pot + ii, V[ii]);
    }
}

int setup_blocks(unsigned long long nvals)
{
    const unsigned long long want = (nvals + 255) / 256;
    const unsigned long long cap = 152ull * 8;  // 8 CTAs of 256 per SM, grid-stride beyond
    return int(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

cudaError_t launch_setup_sample(const SetupGeometry &geo, const double *f, double2 *psi0, double *V,
                                unsigned long long *maxbits, unsigned long long nvals, cudaStream_t s)
{
    setup_sample_kernel<<<setup_blocks(nvals), 256, 0, s>>>(geo, f, psi0, V, maxbits, nvals);
    return cudaGetLastError();
}

cudaError_t launch_setup_noise(int precision, const double2 *psi0, const int2 *noise, const double *V,
                               double amplitude, const double odd_phase[2], void *even, void *odd, void *pot,
                               unsigned long long nvals, cudaStream_t s)
{
    if (precision == GPE_FP64)
        setup_noise_kernel<double><<<setup_blocks(nvals), 256, 0, s>>>(
            psi0, noise, V, amplitude, odd_phase[0], odd_phase[1], (double2 *)even, (double2 *)odd, (double *)pot,
            nvals);
    else
        setup_noise_kernel<float><<<setup_blocks(nvals), 256, 0, s>>>(
            psi0, noise, V, amplitude, odd_phase[0], odd_phase[1], (float2 *)even, (float2 *)odd, (float *)pot,
            nvals);
    return cudaGetLastError();
}

}  // namespace gpe
