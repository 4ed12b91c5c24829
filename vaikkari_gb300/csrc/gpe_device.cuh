// gpe_device.cuh - device-side data layout and the update arithmetic shared by
// every stepping kernel.
//
// Device layout of one field of one instance ("block-ordered structure of
// arrays"): index
//     base + (z+1)*zstride + s*plane + (y+1)*px + (x+kPadX)
// for block (x,y,z), slot s; plane = px*(ny+2), zstride = slots*plane.  Each
// instance carries a ring of zero values around its blocks (one plane below and
// above, one row at each y end, at least one column after x and kPadX = 2
// columns before it, so that interior rows start on a 16-byte boundary for FP32
// pairs).  The zeros are the Dirichlet psi = 0 boundary that the reference gets
// from its padding blocks (GPUGrossPitaevskii_BCC.cu:269-287); they are never
// written, so stencil reads need no bounds checks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gpe {

struct InstDev {
    int nx, ny, nz;   // blocks
    int px, py;       // padded row pitch (elements), padded rows (ny + 2)
    int slots;
    long long plane;   // px * py
    long long zstride; // slots * plane
    long long base;    // element offset of this instance in the field arenas
    long long vbase;   // ARRAY: offset in the potential arena (same layout as a field)
                       // TRAP : offset of the per-axis tables [axis][slot][i]
    double Lc[2];      // -0.5 * w_c * dt     (class weights pre-multiplied by dt)
    double L0;         // 0.5 * dt * sum_k w_k (diagonal term, GPUGrossPitaevskii_BCC.cu:293)
    double gdt;        // g * dt
    double dt, g;
    double vol;        // volume per value
    double w[2];       // unscaled class weights
    // TETRA12 in the face form (gpe_config.faces), per slot s its faces k = 0..3 in
    // summation order at [4 s + k]: packed neighbour (as the lattice tables), the
    // update weight -0.5 hodge / bs^2 * dt in FP64 and FP32, and hodge / bs^2 for
    // the kinetic energy.
    int face;
    int fe[48];
    float hf32[48];
    double hf[48];
    double hw[48];
};

struct WorkItem {
    int inst;
    int x0, y0;
    int z0, z1;
};

// Imaginary-time bookkeeping of one instance (device resident).
struct ImagScalars {
    double sigma;      // scale that normalises the field entering the next step
    double mu;         // chemical potential of the normalised field entering the last step
    double mu_prev;
    double dmu;        // |mu - mu_prev|
    double energy;     // energy of that normalised field
    double norm_in;    // norm of the unscaled field entering the last step
    long long conv_step;  // first step with dmu < tol, -1 while not converged
    long long steps;      // steps taken
};

// Columns of zero padding before x = 0 in every row of the padded layout.  The
// tile boxes start at column x0 - 2 + kPadX (previous field, two-column halo) and
// x0 + kPadX (interior), both 16-byte aligned for any even kPadX.
constexpr int kPadX = 2;

__host__ __device__ inline long long field_index(const InstDev &d, int s, int x, int y, int z)
{
    return d.base + (long long)(z + 1) * d.zstride + (long long)s * d.plane + (long long)(y + 1) * d.px + (x + kPadX);
}

// GPE_FP32C: the residual of the value at field index i is word i - kLoShift of
// the residual array, which puts column x of a row at word x of the row, so a
// tile's residual box starts on the tile's first column (16-byte aligned: rows
// of px = 8k words from an instance base that is a multiple of 64) and is
// exactly the tile wide.  Only interior values (index >= 2 within their row)
// have residuals.
constexpr int kLoShift = kPadX;

#ifdef __CUDACC__
// The digits of a value number v = ((d3 * r2 + d2) * r1 + d1) * r0 + d0, d0
// fastest: in 32-bit division whenever v fits in 31 bits (64-bit division is a
// long instruction sequence on the GPU, 32-bit division a short one).
__device__ __forceinline__ void digits(long long v, int r0, int r1, int r2, int &d0, int &d1, int &d2, int &d3)
{
    if (v <= 0x7fffffffll) {
        unsigned u = unsigned(v);
        d0 = int(u % unsigned(r0));
        u /= unsigned(r0);
        d1 = int(u % unsigned(r1));
        u /= unsigned(r1);
        d2 = int(u % unsigned(r2));
        d3 = int(u / unsigned(r2));
        return;
    }
    long long r = v;
    d0 = int(r % r0);
    r /= r0;
    d1 = int(r % r1);
    r /= r1;
    d2 = int(r % r2);
    d3 = int(r / r2);
}
#endif

#ifdef __CUDACC__
// Rounded arithmetic without contraction, so that the CPU oracle (C fma(),
// -ffp-contract=off) reproduces every result bit for bit.
__device__ __forceinline__ float d_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float d_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float d_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float d_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double d_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double d_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double d_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double d_fma(double a, double b, double c) { return __fma_rn(a, b, c); }

// Packed FP32 pairs (add / mul / fma .rn.f32x2, sm_100 and later): each lane is
// the IEEE operation of that lane, so a complex sum, or a complex times a real
// factor, rounds exactly as the two scalar operations do, in one instruction.
__device__ __forceinline__ float2 f2_add(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "add.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 f2_mul(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 f2_sub(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "sub.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c)
{
    float2 r;
    asm("{\n\t.reg .b64 a, b, c, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mov.b64 c, {%6, %7};\n\tfma.rn.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

template <typename T>
__device__ __forceinline__ typename Cplx<T>::type c_add(typename Cplx<T>::type a, typename Cplx<T>::type b)
{
    typename Cplx<T>::type r;
    r.x = d_add(a.x, b.x);
    r.y = d_add(a.y, b.y);
    return r;
}

template <typename T>
__device__ __forceinline__ typename Cplx<T>::type c_scale(T s, typename Cplx<T>::type a)
{
    typename Cplx<T>::type r;
    r.x = d_mul(s, a.x);
    r.y = d_mul(s, a.y);
    return r;
}

// dt * H psi for one value, given the per-class neighbour sums S[c]
// (each summed in table order).  Restates the arithmetic of the reference's
// update (GPUGrossPitaevskii_BCC.cu:211-213):
//     sum = lapfac * sum_nbr + (lapfac0 + V*dt + g*dt*|psi|^2) * psi
// with one weight per class:
//     nrm = fma(p.x, p.x, p.y*p.y)
//     c   = fma(gdt, nrm, L0 + Vdt)
//     one class:  h = fma(L[0], S[0], c*p)
//     two classes: a = L[0]*S[0], a = fma(L[1], S[1], a), h = fma(c, p, a)
// With BASE, `vdt` already holds L0 + Vdt (rounded the same way, once per
// potential upload) and L0 is not used: one FP64 operation fewer per value.
template <typename T, int NC, bool BASE = false>
__device__ __forceinline__ void hpsi(typename Cplx<T>::type p, const typename Cplx<T>::type *S, const T *L, T L0,
                                     T vdt, T gdt, T &hx, T &hy, T &nrm)
{
    nrm = d_fma(p.x, p.x, d_mul(p.y, p.y));
    const T c = BASE ? d_fma(gdt, nrm, vdt) : d_fma(gdt, nrm, d_add(L0, vdt));
    if (NC == 1) {
        // One class (TETRA12): h = fma(L, S, c*p), the product c*p rounded first.
        // This is the rounding of the reference's update as compiled for the GPU:
        // with it (and the reference's neighbour order) results equal its kernel
        // bit for bit.
        hx = d_fma(L[0], S[0].x, d_mul(c, p.x));
        hy = d_fma(L[0], S[0].y, d_mul(c, p.y));
        return;
    }
    T ax = d_mul(L[0], S[0].x);
    T ay = d_mul(L[0], S[0].y);
#pragma unroll
    for (int k = 1; k < NC; k++) {
        ax = d_fma(L[k], S[k].x, ax);
        ay = d_fma(L[k], S[k].y, ay);
    }
    hx = d_fma(c, p.x, ax);
    hy = d_fma(c, p.y, ay);
}

// Real time: next += -i * h (GPUGrossPitaevskii_BCC.cu:215).
// Imaginary time: next = p - h.
template <typename T, int MODE>
__device__ __forceinline__ typename Cplx<T>::type integrate(typename Cplx<T>::type next, typename Cplx<T>::type p, T hx,
                                                            T hy)
{
    typename Cplx<T>::type r;
    if (MODE == 0) {
        r.x = d_add(next.x, hy);
        r.y = d_sub(next.y, hx);
    } else {
        r.x = d_sub(p.x, hx);
        r.y = d_sub(p.y, hy);
    }
    return r;
}

// Compensated storage (GPE_FP32C): each component of a stored FP32 value s
// carries an int8 residual q in units of ulp(s)/256, so the value stands for
// s + q * unit(s).  unit(s) = 2^(E - 31 - 127) for the biased exponent E of s,
// with E raised to 32 below 2^-95 so that the unit stays a normal float.  A
// two-sum's rounding error is at most ulp(s)/2 = 128 units: q is the error in
// units rounded to nearest even and clipped to +-127.  Scaling by a power of
// two is exact, so encoding and decoding round only in that one place.
__device__ __forceinline__ float comp_unit(float s)
{
    const uint32_t e = max(__float_as_uint(s) & 0x7f800000u, 32u << 23);
    return __uint_as_float(e - (31u << 23));
}
__device__ __forceinline__ float comp_unit_inv(float s)  // 1 / comp_unit(s), exactly
{
    const uint32_t e = max(__float_as_uint(s) & 0x7f800000u, 32u << 23);
    return __uint_as_float((285u << 23) - e);
}
__device__ __forceinline__ uint32_t comp_encode(float r, float s)  // the low 8 bits hold q
{
    const int q = min(max(__float2int_rn(__fmul_rn(r, comp_unit_inv(s))), -127), 127);
    return uint32_t(q) & 0xffu;
}
__device__ __forceinline__ float comp_decode(uint32_t q8, float s)
{
    return __fmul_rn(float(int(int8_t(uint8_t(q8)))), comp_unit(s));
}

// Harmonic trap from per-axis tables (dt-scaled): V = (Vx + Vy) + Vz.
template <typename T>
__device__ __forceinline__ T trap_vdt(const T *tab, const InstDev &d, int s, int x, int y, int z)
{
    const T *tx = tab + d.vbase;
    const T *ty = tx + (long long)d.slots * d.nx;
    const T *tz = ty + (long long)d.slots * d.ny;
    return d_add(d_add(tx[s * d.nx + x], ty[s * d.ny + y]), tz[s * d.nz + z]);
}
#endif  // __CUDACC__

}  // namespace gpe
