/*
 * gpe_oracle.h - CPU oracle for the GPE stepper.  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
 * check the library's results; never part of the shipped library.
 *
 * A plain-C restatement of the reference's algorithm
 * (markus-kivioja/vaikkari, koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu):
 *   - update():        :176-216 (neighbour sum, potential, nonlinearity, next -= i*sum)
 *   - dt scaling:      :289-307 (lapfac = -0.5*hodge/bs^2*dt, lapfac0 = -sum(lapfac))
 *   - leapfrog order:  :475-481 (odd <- even, then even <- odd)
 *   - zero padding:    :269-287 (psi = 0 outside the block grid)
 * over a generic neighbour table (the reference's 48-entry table of :90-142, or
 * the 14-edge BCC table), and the face form of the multi-GPU program's update
 * (GPUGrossPitaevskii_BCC_multi.cu:329-397); the imaginary-time step and the observables have no
 * counterpart in the reference and are restated from their definitions.
 *
 * Layout: the reference's block order, index (((z*ny)+y)*nx+x)*slots+s;
 * complex values interleaved (re, im).
 *
 * The _f32 functions perform exactly the rounded operations of the GPU kernels
 * (fmaf/multiply/add in the same order, no contraction), so the GPU FP32 path
 * can be compared bit for bit; the _f64 functions do the same in double.
 */
#ifndef GPE_ORACLE_H
#define GPE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_grid {
    int nx, ny, nz;
    int slots, neighbours;
    const int *entry;   /* slots*neighbours*5: (dx, dy, dz, slot, class), classes ascending per slot */
    double Lc[2];       /* -0.5 * w_c * dt */
    double L0;          /* 0.5 * dt * sum of weights */
    double gdt;         /* g * dt */
} oracle_grid;

/* One half-step.  mode 0: next += -i*h(prev); mode 1: next = p - h(p) with
 * p = sigma*prev (imaginary time).  vdt = V*dt per value. */
void oracle_half_step_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt, int mode,
                          double sigma);
void oracle_half_step_f32(const oracle_grid *g, const float *prev, float *next, const float *vdt, int mode,
                          float sigma);

/* BCC2 lattice only, in the summation order of the fused GPU kernel, which
 * reuses 2x2 diagonal box sums and axial pair sums across planes.  With
 * C = slot 0 (cube corner), B = slot 1 (cube centre), zero outside the grid,
 * every value pre-multiplied by sigma in imaginary time:
 *   bB(x,y,q) = (B(x-1,y-1,q) + B(x,y-1,q)) + (B(x-1,y,q) + B(x,y,q))
 *   bC(x,y,q) = (C(x,y,q) + C(x+1,y,q)) + (C(x,y+1,q) + C(x+1,y+1,q))
 *   slot 0:  Sd = bB(z-1) + bB(z)
 *            Sa = (C(z-1) + C(z+1)) + ((C(x-1) + C(x+1)) + (C(y-1) + C(y+1)))
 *   slot 1:  Sd = bC(z) + bC(z+1)
 *            Sa = (B(z-1) + B(z+1)) + ((B(x-1) + B(x+1)) + (B(y-1) + B(y+1)))
 * then the same h and integrator as oracle_half_step_*. */
void oracle_half_step_bcc2_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt, int mode,
                               double sigma);
void oracle_half_step_bcc2_f32(const oracle_grid *g, const float *prev, float *next, const float *vdt, int mode,
                               float sigma);
void oracle_leapfrog_bcc2_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps);
void oracle_leapfrog_bcc2_f32(const oracle_grid *g, float *even, float *odd, const float *vdt, long steps);
/* BCC2 real time with compensated storage: next += -i h as an exact two-sum of
 * the stored FP32 value and (residual + increment); the rounding error is kept
 * as an int8 residual per component in units of ulp/256 (re, im per value, block order). */
void oracle_half_step_bcc2_f32c(const oracle_grid *g, const float *prev, float *next, int8_t *next_lo,
                                const float *vdt);
void oracle_leapfrog_bcc2_f32c(const oracle_grid *g, float *even, float *odd, int8_t *even_lo, int8_t *odd_lo,
                               const float *vdt, long steps);

/* The BCC2 real-time half-step/leapfrog with direct indexing for interior values
 * (bit-identical to the _bcc2_ functions); the timed CPU baseline. */
void oracle_half_step_bcc2_fast_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt,
                                    int mode, double sigma);
void oracle_leapfrog_bcc2_fast_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps);

/* `steps` leapfrog steps (odd <- even, even <- odd). */
void oracle_leapfrog_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps);
void oracle_leapfrog_f32(const oracle_grid *g, float *even, float *odd, const float *vdt, long steps);

/* Sums over values (no volume factor), Kahan-compensated, sequential order:
 * out[0] = |psi|^2, out[1] = Re(conj(psi) * (-1/2 Lap psi)), out[2] = V|psi|^2,
 * out[3] = g/2 |psi|^4.  w = unscaled class weights; vdt/dt recovers V. */
void oracle_observables_f64(const oracle_grid *g, const double *psi, const double *vdt, double dt, double gcoef,
                            const double *w, double *out);
void oracle_observables_f32(const oracle_grid *g, const float *psi, const float *vdt, double dt, double gcoef,
                            const double *w, double *out);

/* Imaginary time in FP64: `steps` normalised Euler steps of psi (psi and work
 * ping-pong; the result ends in psi, normalised).  mu_hist[k] (may be NULL)
 * receives mu of the normalised field entering step k.  Returns the first step
 * with |mu_k - mu_{k-1}| < tol, or -1.  vol = volume per value. */
long oracle_imaginary_f64(const oracle_grid *g, double *psi, double *work, const double *vdt, double dt,
                          double gcoef, const double *w, double vol, long steps, double tol, double *mu_hist);

/* The face (Hodge) form of the reference's multi-GPU update
 * (GPUGrossPitaevskii_BCC_multi.cu:329-397) on a 12-slot grid: per value, over
 * its four faces in summation order (face[(s*4+k)*4 ..] = dx, dy, dz, slot;
 * h[s*4+k] = -0.5 * hodge / bs^2 * dt), zero outside the grid,
 *   sum = fma(h_k, psi_k - psi, sum)            k = 0..3, from sum = 0
 *   sum = fma(fma(gdt, fma(x, x, y*y), vdt), psi, sum)
 *   mode 0: next += -i sum;  mode 1: next = psi - sum, psi = sigma * prev.
 * These are the roundings of that kernel as nvcc compiles it. */
void oracle_half_step_faces_f64(int nx, int ny, int nz, const int *face, const double *h, double gdt,
                                const double *prev, double *next, const double *vdt, int mode, double sigma);
void oracle_half_step_faces_f32(int nx, int ny, int nz, const int *face, const float *h, float gdt,
                                const float *prev, float *next, const float *vdt, int mode, float sigma);
void oracle_leapfrog_faces_f64(int nx, int ny, int nz, const int *face, const double *h, double gdt, double *even,
                               double *odd, const double *vdt, long steps);
void oracle_leapfrog_faces_f32(int nx, int ny, int nz, const int *face, const float *h, float gdt, float *even,
                               float *odd, const float *vdt, long steps);

/* Worker threads used by the parallel loops (OpenMP). */
void oracle_set_threads(int n);
int oracle_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
