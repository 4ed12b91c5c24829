/*
 * gpe_oracle.c - CPU oracle for the GPE stepper (test infrastructure only; see
 * gpe_oracle.h).  Build: make -C oracle oracle  (or vaikkari_gb300.build), with
 * -ffp-contract=off so that a*b+c is never fused behind our back: every fused
 * multiply-add below is an explicit fma()/fmaf(), matching the GPU kernels.
 */
#include "gpe_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void oracle_set_threads(int n) { g_threads = n; }
int oracle_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* Compensated storage (GPE_FP32C): the residual of a stored FP32 value s as an
 * int8 q in units of ulp(s)/256.  unit(s) = 2^(E - 31 - 127) for the biased
 * exponent E of s, E raised to 32 below 2^-95; q = the residual in units,
 * rounded to nearest even (rintf in the default rounding mode) and clipped to
 * +-127.  Scaling by the power of two unit(s) is exact. */
static inline float comp_unit(float s)
{
    uint32_t u;
    memcpy(&u, &s, 4);
    u &= 0x7f800000u;
    if (u < (32u << 23)) u = 32u << 23;
    u -= 31u << 23;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline int8_t comp_encode(float r, float s)
{
    float q = rintf(r / comp_unit(s));
    if (q > 127.0f) q = 127.0f;
    if (q < -127.0f) q = -127.0f;
    return (int8_t)q;
}
static inline float comp_decode(int8_t q, float s) { return (float)q * comp_unit(s); }

#define IDX(g, x, y, z, s) (((((size_t)(z) * (g)->ny) + (size_t)(y)) * (g)->nx + (size_t)(x)) * (g)->slots + (size_t)(s))

/*
 * The per-value update, GPUGrossPitaevskii_BCC.cu:207-215:
 *   sum  = lapfac * (n0 + n1 + n2 + n3) + (lapfac0 + pot + g*|prev|^2) * prev
 *   next += (sum.y, -sum.x)
 * generalised to per-class neighbour sums S[c] and weights Lc[c]:
 *   nrm = fma(p.x, p.x, p.y*p.y);  c = fma(gdt, nrm, L0 + vdt)
 *   a   = Lc[0]*S[0] (then a = fma(Lc[c], S[c], a));  h = fma(c, p, a)
 * Out-of-grid neighbours are zero (the reference's padding blocks, :269-287).
 */
#define HALF_STEP_BODY(T, FMA)                                                                      \
    const int ns = g->slots, nb = g->neighbours;                                                   \
    const T L0 = (T)g->L0, gdt = (T)g->gdt;                                                         \
    const T Lc0 = (T)g->Lc[0], Lc1 = (T)g->Lc[1];                                                   \
    int z;                                                                                          \
    _Pragma("omp parallel for schedule(static) num_threads(oracle_get_threads())")                  \
    for (z = 0; z < g->nz; z++) {                                                                   \
        for (int y = 0; y < g->ny; y++)                                                             \
            for (int x = 0; x < g->nx; x++)                                                         \
                for (int s = 0; s < ns; s++) {                                                      \
                    T sx[2] = {0, 0}, sy[2] = {0, 0};                                               \
                    int seen[2] = {0, 0};                                                           \
                    int ncls = 1;                                                                   \
                    for (int k = 0; k < nb; k++) {                                                  \
                        const int *e = g->entry + ((size_t)s * nb + k) * 5;                         \
                        const int xx = x + e[0], yy = y + e[1], zz = z + e[2], c = e[4];            \
                        T vx = 0, vy = 0;                                                           \
                        if (xx >= 0 && xx < g->nx && yy >= 0 && yy < g->ny && zz >= 0 && zz < g->nz) { \
                            const size_t o = IDX(g, xx, yy, zz, e[3]);                              \
                            vx = prev[2 * o];                                                       \
                            vy = prev[2 * o + 1];                                                   \
                            if (mode == 1) {                                                        \
                                vx = sigma * vx;                                                    \
                                vy = sigma * vy;                                                    \
                            }                                                                       \
                        }                                                                           \
                        if (c + 1 > ncls) ncls = c + 1;                                             \
                        if (!seen[c]) {                                                             \
                            sx[c] = vx;                                                             \
                            sy[c] = vy;                                                             \
                            seen[c] = 1;                                                            \
                        } else {                                                                    \
                            sx[c] = sx[c] + vx;                                                     \
                            sy[c] = sy[c] + vy;                                                     \
                        }                                                                           \
                    }                                                                               \
                    const size_t o = IDX(g, x, y, z, s);                                            \
                    T px = prev[2 * o], py = prev[2 * o + 1];                                       \
                    if (mode == 1) {                                                                \
                        px = sigma * px;                                                            \
                        py = sigma * py;                                                            \
                    }                                                                               \
                    const T nrm = FMA(px, px, py * py);                                             \
                    const T cc = FMA(gdt, nrm, L0 + vdt[o]);                                        \
                    T hx, hy;                                                                       \
                    if (ncls == 1) { /* one class: fma(L, S, c*p), the reference kernel's rounding */ \
                        hx = FMA(Lc0, sx[0], cc * px);                                              \
                        hy = FMA(Lc0, sy[0], cc * py);                                              \
                    } else {                                                                        \
                        const T ax = FMA(Lc1, sx[1], Lc0 * sx[0]), ay = FMA(Lc1, sy[1], Lc0 * sy[0]); \
                        hx = FMA(cc, px, ax);                                                       \
                        hy = FMA(cc, py, ay);                                                       \
                    }                                                                               \
                    if (mode == 0) {                                                                \
                        next[2 * o] = next[2 * o] + hy;                                             \
                        next[2 * o + 1] = next[2 * o + 1] - hx;                                     \
                    } else {                                                                        \
                        next[2 * o] = px - hx;                                                      \
                        next[2 * o + 1] = py - hy;                                                  \
                    }                                                                               \
                }                                                                                   \
    }

void oracle_half_step_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt, int mode,
                          double sigma)
{
    HALF_STEP_BODY(double, fma)
}

void oracle_half_step_f32(const oracle_grid *g, const float *prev, float *next, const float *vdt, int mode,
                          float sigma)
{
    HALF_STEP_BODY(float, fmaf)
}

/* GPUGrossPitaevskii_BCC.cu:475-481: update odd from even, then even from odd. */
void oracle_leapfrog_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_f64(g, even, odd, vdt, 0, 1.0);
        oracle_half_step_f64(g, odd, even, vdt, 0, 1.0);
    }
}

void oracle_leapfrog_f32(const oracle_grid *g, float *even, float *odd, const float *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_f32(g, even, odd, vdt, 0, 1.0f);
        oracle_half_step_f32(g, odd, even, vdt, 0, 1.0f);
    }
}

/* The face form of GPUGrossPitaevskii_BCC_multi.cu:329-397 (see gpe_oracle.h). */
#define FIDX(x, y, z, s) ((((size_t)(z) * (size_t)ny + (size_t)(y)) * (size_t)nx + (size_t)(x)) * 12 + (size_t)(s))
#define FACES_BODY(T, FMA)                                                                          \
    int z;                                                                                          \
    _Pragma("omp parallel for schedule(static) num_threads(oracle_get_threads())")                  \
    for (z = 0; z < nz; z++) {                                                                      \
        for (int y = 0; y < ny; y++)                                                                \
            for (int x = 0; x < nx; x++)                                                            \
                for (int s = 0; s < 12; s++) {                                                      \
                    const size_t o = FIDX(x, y, z, s);                                              \
                    T px = prev[2 * o], py = prev[2 * o + 1];                                       \
                    if (mode == 1) {                                                                \
                        px = sigma * px;                                                            \
                        py = sigma * py;                                                            \
                    }                                                                               \
                    T sx = 0, sy = 0;                                                               \
                    for (int k = 0; k < 4; k++) {                                                   \
                        const int *e = face + (s * 4 + k) * 4;                                      \
                        const int xx = x + e[0], yy = y + e[1], zz = z + e[2];                      \
                        T vx = 0, vy = 0;                                                           \
                        if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) {       \
                            const size_t q = FIDX(xx, yy, zz, e[3]);                                \
                            vx = prev[2 * q];                                                       \
                            vy = prev[2 * q + 1];                                                   \
                            if (mode == 1) {                                                        \
                                vx = sigma * vx;                                                    \
                                vy = sigma * vy;                                                    \
                            }                                                                       \
                        }                                                                           \
                        sx = FMA(h[s * 4 + k], vx - px, sx);                                        \
                        sy = FMA(h[s * 4 + k], vy - py, sy);                                        \
                    }                                                                               \
                    const T cc = FMA(gdt, FMA(px, px, py * py), vdt[o]);                            \
                    sx = FMA(cc, px, sx);                                                           \
                    sy = FMA(cc, py, sy);                                                           \
                    if (mode == 0) {                                                                \
                        next[2 * o] = next[2 * o] + sy;                                             \
                        next[2 * o + 1] = next[2 * o + 1] - sx;                                     \
                    } else {                                                                        \
                        next[2 * o] = px - sx;                                                      \
                        next[2 * o + 1] = py - sy;                                                  \
                    }                                                                               \
                }                                                                                   \
    }

void oracle_half_step_faces_f64(int nx, int ny, int nz, const int *face, const double *h, double gdt,
                                const double *prev, double *next, const double *vdt, int mode, double sigma)
{
    FACES_BODY(double, fma)
}

void oracle_half_step_faces_f32(int nx, int ny, int nz, const int *face, const float *h, float gdt,
                                const float *prev, float *next, const float *vdt, int mode, float sigma)
{
    FACES_BODY(float, fmaf)
}

void oracle_leapfrog_faces_f64(int nx, int ny, int nz, const int *face, const double *h, double gdt, double *even,
                               double *odd, const double *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_faces_f64(nx, ny, nz, face, h, gdt, even, odd, vdt, 0, 1.0);
        oracle_half_step_faces_f64(nx, ny, nz, face, h, gdt, odd, even, vdt, 0, 1.0);
    }
}

void oracle_leapfrog_faces_f32(int nx, int ny, int nz, const int *face, const float *h, float gdt, float *even,
                               float *odd, const float *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_faces_f32(nx, ny, nz, face, h, gdt, even, odd, vdt, 0, 1.0f);
        oracle_half_step_faces_f32(nx, ny, nz, face, h, gdt, odd, even, vdt, 0, 1.0f);
    }
}

/* BCC2 in the fused kernel's order (see gpe_oracle.h). */
#define BCC2_BODY(T, FMA)                                                                           \
    const int nx = g->nx, ny = g->ny, nz = g->nz;                                                  \
    const T L0 = (T)g->L0, gdt = (T)g->gdt;                                                         \
    const T Lc0 = (T)g->Lc[0], Lc1 = (T)g->Lc[1];                                                   \
    int z;                                                                                          \
    _Pragma("omp parallel for schedule(static) num_threads(oracle_get_threads())")                  \
    for (z = 0; z < nz; z++) {                                                                      \
        for (int y = 0; y < ny; y++)                                                                \
            for (int x = 0; x < nx; x++) {                                                          \
                T vx[2][3][3][3], vy[2][3][3][3]; /* [slot][dz+1][dy+1][dx+1] */                    \
                for (int s = 0; s < 2; s++)                                                         \
                    for (int dz = -1; dz <= 1; dz++)                                                \
                        for (int dy = -1; dy <= 1; dy++)                                            \
                            for (int dx = -1; dx <= 1; dx++) {                                      \
                                const int xx = x + dx, yy = y + dy, zz = z + dz;                    \
                                T a = 0, b = 0;                                                     \
                                if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) { \
                                    const size_t o = IDX(g, xx, yy, zz, s);                         \
                                    a = prev[2 * o];                                                \
                                    b = prev[2 * o + 1];                                            \
                                    if (mode == 1) {                                                \
                                        a = sigma * a;                                              \
                                        b = sigma * b;                                              \
                                    }                                                               \
                                }                                                                   \
                                vx[s][dz + 1][dy + 1][dx + 1] = a;                                  \
                                vy[s][dz + 1][dy + 1][dx + 1] = b;                                  \
                            }                                                                       \
                for (int s = 0; s < 2; s++) {                                                       \
                    T sdx, sdy, sax, say;                                                           \
                    const T(*X)[3][3] = vx[s];                                                      \
                    const T(*Y)[3][3] = vy[s];                                                      \
                    const T(*OX)[3][3] = vx[1 - s];                                                 \
                    const T(*OY)[3][3] = vy[1 - s];                                                 \
                    if (s == 0) { /* boxes of B at planes z-1, z around (x-1..x, y-1..y) */         \
                        const T b0x = (OX[0][0][0] + OX[0][0][1]) + (OX[0][1][0] + OX[0][1][1]);    \
                        const T b0y = (OY[0][0][0] + OY[0][0][1]) + (OY[0][1][0] + OY[0][1][1]);    \
                        const T b1x = (OX[1][0][0] + OX[1][0][1]) + (OX[1][1][0] + OX[1][1][1]);    \
                        const T b1y = (OY[1][0][0] + OY[1][0][1]) + (OY[1][1][0] + OY[1][1][1]);    \
                        sdx = b0x + b1x;                                                            \
                        sdy = b0y + b1y;                                                            \
                    } else { /* boxes of C at planes z, z+1 around (x..x+1, y..y+1) */              \
                        const T b0x = (OX[1][1][1] + OX[1][1][2]) + (OX[1][2][1] + OX[1][2][2]);    \
                        const T b0y = (OY[1][1][1] + OY[1][1][2]) + (OY[1][2][1] + OY[1][2][2]);    \
                        const T b1x = (OX[2][1][1] + OX[2][1][2]) + (OX[2][2][1] + OX[2][2][2]);    \
                        const T b1y = (OY[2][1][1] + OY[2][1][2]) + (OY[2][2][1] + OY[2][2][2]);    \
                        sdx = b0x + b1x;                                                            \
                        sdy = b0y + b1y;                                                            \
                    }                                                                               \
                    sax = (X[0][1][1] + X[2][1][1]) + ((X[1][1][0] + X[1][1][2]) + (X[1][0][1] + X[1][2][1])); \
                    say = (Y[0][1][1] + Y[2][1][1]) + ((Y[1][1][0] + Y[1][1][2]) + (Y[1][0][1] + Y[1][2][1])); \
                    const T px = X[1][1][1], py = Y[1][1][1];                                       \
                    const size_t o = IDX(g, x, y, z, s);                                            \
                    const T nrm = FMA(px, px, py * py);                                             \
                    const T cc = FMA(gdt, nrm, L0 + vdt[o]);                                        \
                    T ax = Lc0 * sdx, ay = Lc0 * sdy;                                               \
                    ax = FMA(Lc1, sax, ax);                                                         \
                    ay = FMA(Lc1, say, ay);                                                         \
                    const T hx = FMA(cc, px, ax), hy = FMA(cc, py, ay);                             \
                    if (mode == 0 && next_lo) { /* compensated storage: exact two-sum */            \
                        const T ux = next[2 * o], uy = next[2 * o + 1];                             \
                        const T tx = (T)comp_decode(next_lo[2 * o], (float)ux) + hy;                \
                        const T ty = (T)comp_decode(next_lo[2 * o + 1], (float)uy) - hx;            \
                        const T wx = ux + tx, wy = uy + ty;                                         \
                        const T bx = wx - ux, by = wy - uy;                                         \
                        const T rx = (ux - (wx - bx)) + (tx - bx);                                  \
                        const T ry = (uy - (wy - by)) + (ty - by);                                  \
                        next[2 * o] = wx;                                                           \
                        next[2 * o + 1] = wy;                                                       \
                        next_lo[2 * o] = comp_encode((float)rx, (float)wx);                         \
                        next_lo[2 * o + 1] = comp_encode((float)ry, (float)wy);                     \
                    } else if (mode == 0) {                                                         \
                        next[2 * o] = next[2 * o] + hy;                                             \
                        next[2 * o + 1] = next[2 * o + 1] - hx;                                     \
                    } else {                                                                        \
                        next[2 * o] = px - hx;                                                      \
                        next[2 * o + 1] = py - hy;                                                  \
                    }                                                                               \
                }                                                                                   \
            }                                                                                       \
    }

void oracle_half_step_bcc2_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt, int mode,
                               double sigma)
{
    int8_t *const next_lo = NULL;
    BCC2_BODY(double, fma)
}

/* One value of the checked BCC2 path (both slots of block (x, y, z)). */
static void bcc2_value_f64(const oracle_grid *g0, const double *prev, double *next, const double *vdt, int mode,
                           double sigma, int x0, int y0, int z0)
{
    oracle_grid one = *g0;
    /* run the checked body on a 1x1x1 window by offsetting the loops */
#define T double
#define FMA fma
    const oracle_grid *g = g0;
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const T L0 = (T)g->L0, gdt = (T)g->gdt;
    const T Lc0 = (T)g->Lc[0], Lc1 = (T)g->Lc[1];
    (void)one;
    {
        const int z = z0, y = y0, x = x0;
        T vx[2][3][3][3], vy[2][3][3][3];
        for (int s = 0; s < 2; s++)
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int xx = x + dx, yy = y + dy, zz = z + dz;
                        T a = 0, b = 0;
                        if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) {
                            const size_t o = IDX(g, xx, yy, zz, s);
                            a = prev[2 * o];
                            b = prev[2 * o + 1];
                            if (mode == 1) {
                                a = sigma * a;
                                b = sigma * b;
                            }
                        }
                        vx[s][dz + 1][dy + 1][dx + 1] = a;
                        vy[s][dz + 1][dy + 1][dx + 1] = b;
                    }
        for (int s = 0; s < 2; s++) {
            T sdx, sdy, sax, say;
            const T(*X)[3][3] = vx[s];
            const T(*Y)[3][3] = vy[s];
            const T(*OX)[3][3] = vx[1 - s];
            const T(*OY)[3][3] = vy[1 - s];
            if (s == 0) {
                const T b0x = (OX[0][0][0] + OX[0][0][1]) + (OX[0][1][0] + OX[0][1][1]);
                const T b0y = (OY[0][0][0] + OY[0][0][1]) + (OY[0][1][0] + OY[0][1][1]);
                const T b1x = (OX[1][0][0] + OX[1][0][1]) + (OX[1][1][0] + OX[1][1][1]);
                const T b1y = (OY[1][0][0] + OY[1][0][1]) + (OY[1][1][0] + OY[1][1][1]);
                sdx = b0x + b1x;
                sdy = b0y + b1y;
            } else {
                const T b0x = (OX[1][1][1] + OX[1][1][2]) + (OX[1][2][1] + OX[1][2][2]);
                const T b0y = (OY[1][1][1] + OY[1][1][2]) + (OY[1][2][1] + OY[1][2][2]);
                const T b1x = (OX[2][1][1] + OX[2][1][2]) + (OX[2][2][1] + OX[2][2][2]);
                const T b1y = (OY[2][1][1] + OY[2][1][2]) + (OY[2][2][1] + OY[2][2][2]);
                sdx = b0x + b1x;
                sdy = b0y + b1y;
            }
            sax = (X[0][1][1] + X[2][1][1]) + ((X[1][1][0] + X[1][1][2]) + (X[1][0][1] + X[1][2][1]));
            say = (Y[0][1][1] + Y[2][1][1]) + ((Y[1][1][0] + Y[1][1][2]) + (Y[1][0][1] + Y[1][2][1]));
            const T px = X[1][1][1], py = Y[1][1][1];
            const size_t o = IDX(g, x, y, z, s);
            const T nrm = FMA(px, px, py * py);
            const T cc = FMA(gdt, nrm, L0 + vdt[o]);
            T ax = Lc0 * sdx, ay = Lc0 * sdy;
            ax = FMA(Lc1, sax, ax);
            ay = FMA(Lc1, say, ay);
            const T hx = FMA(cc, px, ax), hy = FMA(cc, py, ay);
            if (mode == 0) {
                next[2 * o] = next[2 * o] + hy;
                next[2 * o + 1] = next[2 * o + 1] - hx;
            } else {
                next[2 * o] = px - hx;
                next[2 * o + 1] = py - hy;
            }
        }
    }
#undef T
#undef FMA
}

void oracle_half_step_bcc2_f32(const oracle_grid *g, const float *prev, float *next, const float *vdt, int mode,
                               float sigma)
{
    int8_t *const next_lo = NULL;
    BCC2_BODY(float, fmaf)
}

/* Real time with compensated storage (GPE_FP32C): next_lo holds the int8
 * residual of each component (comp_encode), (re, im) per value in block order. */
void oracle_half_step_bcc2_f32c(const oracle_grid *g, const float *prev, float *next, int8_t *next_lo,
                                const float *vdt)
{
    const int mode = 0;
    const float sigma = 1.0f;
    (void)sigma;
    BCC2_BODY(float, fmaf)
}

void oracle_leapfrog_bcc2_f32c(const oracle_grid *g, float *even, float *odd, int8_t *even_lo, int8_t *odd_lo,
                               const float *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_bcc2_f32c(g, even, odd, odd_lo, vdt);
        oracle_half_step_bcc2_f32c(g, odd, even, even_lo, vdt);
    }
}

/*
 * The same BCC2 half-step, fast: interior values (one block away from every
 * face) read their 3x3x3 neighbourhood by direct offsets, boundary values take
 * the checked path above.  Same rounded operations in the same order, so it is
 * bit-identical to oracle_half_step_bcc2_f64 (tests check it); used to time the
 * CPU baseline.
 */
static void bcc2_value_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt, int mode,
                           double sigma, int x, int y, int z);

void oracle_half_step_bcc2_fast_f64(const oracle_grid *g, const double *prev, double *next, const double *vdt,
                                    int mode, double sigma)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double L0 = g->L0, gdt = g->gdt, Lc0 = g->Lc[0], Lc1 = g->Lc[1];
    const ptrdiff_t sx = 2, sy = (ptrdiff_t)nx * 2, sz = (ptrdiff_t)nx * ny * 2; /* in slot units */
    int z;
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
    for (z = 0; z < nz; z++) {
        for (int y = 0; y < ny; y++) {
            const int interior_zy = (z > 0 && z < nz - 1 && y > 0 && y < ny - 1);
            for (int x = 0; x < nx; x++) {
                if (!interior_zy || x == 0 || x == nx - 1 || mode != 0) {
                    bcc2_value_f64(g, prev, next, vdt, mode, sigma, x, y, z);
                    continue;
                }
                const ptrdiff_t c = (((ptrdiff_t)z * ny + y) * nx + x) * 2; /* slot-0 index */
#define P(o, s) (prev + 2 * (c + (o) + (s)))
                /* slot 0 (C): B boxes at z-1, z around (x-1..x, y-1..y) */
                {
                    const double *b00 = P(-sz - sy - sx, 1), *b01 = P(-sz - sy, 1), *b02 = P(-sz - sx, 1), *b03 = P(-sz, 1);
                    const double *b10 = P(-sy - sx, 1), *b11 = P(-sy, 1), *b12 = P(-sx, 1), *b13 = P(0, 1);
                    const double sdx = ((b00[0] + b01[0]) + (b02[0] + b03[0])) + ((b10[0] + b11[0]) + (b12[0] + b13[0]));
                    const double sdy = ((b00[1] + b01[1]) + (b02[1] + b03[1])) + ((b10[1] + b11[1]) + (b12[1] + b13[1]));
                    const double *zm = P(-sz, 0), *zp = P(sz, 0), *xm = P(-sx, 0), *xp = P(sx, 0), *ym = P(-sy, 0), *yp = P(sy, 0);
                    const double sax = (zm[0] + zp[0]) + ((xm[0] + xp[0]) + (ym[0] + yp[0]));
                    const double say = (zm[1] + zp[1]) + ((xm[1] + xp[1]) + (ym[1] + yp[1]));
                    const double *p = P(0, 0);
                    const double px = p[0], py = p[1];
                    const double nrm = fma(px, px, py * py);
                    const double cc = fma(gdt, nrm, L0 + vdt[c]);
                    const double ax = fma(Lc1, sax, Lc0 * sdx), ay = fma(Lc1, say, Lc0 * sdy);
                    const double hx = fma(cc, px, ax), hy = fma(cc, py, ay);
                    next[2 * c] = next[2 * c] + hy;
                    next[2 * c + 1] = next[2 * c + 1] - hx;
                }
                /* slot 1 (B): C boxes at z, z+1 around (x..x+1, y..y+1) */
                {
                    const double *c00 = P(0, 0), *c01 = P(sx, 0), *c02 = P(sy, 0), *c03 = P(sy + sx, 0);
                    const double *c10 = P(sz, 0), *c11 = P(sz + sx, 0), *c12 = P(sz + sy, 0), *c13 = P(sz + sy + sx, 0);
                    const double sdx = ((c00[0] + c01[0]) + (c02[0] + c03[0])) + ((c10[0] + c11[0]) + (c12[0] + c13[0]));
                    const double sdy = ((c00[1] + c01[1]) + (c02[1] + c03[1])) + ((c10[1] + c11[1]) + (c12[1] + c13[1]));
                    const double *zm = P(-sz, 1), *zp = P(sz, 1), *xm = P(-sx, 1), *xp = P(sx, 1), *ym = P(-sy, 1), *yp = P(sy, 1);
                    const double sax = (zm[0] + zp[0]) + ((xm[0] + xp[0]) + (ym[0] + yp[0]));
                    const double say = (zm[1] + zp[1]) + ((xm[1] + xp[1]) + (ym[1] + yp[1]));
                    const double *p = P(0, 1);
                    const double px = p[0], py = p[1];
                    const double nrm = fma(px, px, py * py);
                    const double cc = fma(gdt, nrm, L0 + vdt[c + 1]);
                    const double ax = fma(Lc1, sax, Lc0 * sdx), ay = fma(Lc1, say, Lc0 * sdy);
                    const double hx = fma(cc, px, ax), hy = fma(cc, py, ay);
                    next[2 * (c + 1)] = next[2 * (c + 1)] + hy;
                    next[2 * (c + 1) + 1] = next[2 * (c + 1) + 1] - hx;
                }
#undef P
            }
        }
    }
}

void oracle_leapfrog_bcc2_fast_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_bcc2_fast_f64(g, even, odd, vdt, 0, 1.0);
        oracle_half_step_bcc2_fast_f64(g, odd, even, vdt, 0, 1.0);
    }
}

void oracle_leapfrog_bcc2_f64(const oracle_grid *g, double *even, double *odd, const double *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_bcc2_f64(g, even, odd, vdt, 0, 1.0);
        oracle_half_step_bcc2_f64(g, odd, even, vdt, 0, 1.0);
    }
}

void oracle_leapfrog_bcc2_f32(const oracle_grid *g, float *even, float *odd, const float *vdt, long steps)
{
    for (long k = 0; k < steps; k++) {
        oracle_half_step_bcc2_f32(g, even, odd, vdt, 0, 1.0f);
        oracle_half_step_bcc2_f32(g, odd, even, vdt, 0, 1.0f);
    }
}

typedef struct {
    double s, c;
} kahan_t;

static void kahan_add(kahan_t *k, double v)
{
    const double y = v - k->c;
    const double t = k->s + y;
    k->c = (t - k->s) - y;
    k->s = t;
}

#define OBSERVABLES_BODY(T)                                                                          \
    const int ns = g->slots, nb = g->neighbours;                                                    \
    double wsum = 0.0;                                                                               \
    for (int k = 0; k < nb; k++) wsum += w[g->entry[k * 5 + 4]];                                     \
    kahan_t k0 = {0, 0}, k1 = {0, 0}, k2 = {0, 0}, k3 = {0, 0};                                      \
    for (int z = 0; z < g->nz; z++)                                                                  \
        for (int y = 0; y < g->ny; y++)                                                              \
            for (int x = 0; x < g->nx; x++)                                                          \
                for (int s = 0; s < ns; s++) {                                                       \
                    double lx = 0.0, ly = 0.0;                                                       \
                    for (int k = 0; k < nb; k++) {                                                   \
                        const int *e = g->entry + ((size_t)s * nb + k) * 5;                          \
                        const int xx = x + e[0], yy = y + e[1], zz = z + e[2];                       \
                        if (xx < 0 || xx >= g->nx || yy < 0 || yy >= g->ny || zz < 0 || zz >= g->nz) \
                            continue;                                                                \
                        const size_t o = IDX(g, xx, yy, zz, e[3]);                                   \
                        lx += w[e[4]] * (double)psi[2 * o];                                          \
                        ly += w[e[4]] * (double)psi[2 * o + 1];                                      \
                    }                                                                                \
                    const size_t o = IDX(g, x, y, z, s);                                             \
                    const double px = (double)psi[2 * o], py = (double)psi[2 * o + 1];               \
                    lx -= wsum * px;                                                                 \
                    ly -= wsum * py;                                                                 \
                    const double n2 = px * px + py * py;                                             \
                    kahan_add(&k0, n2);                                                              \
                    kahan_add(&k1, -0.5 * (px * lx + py * ly));                                      \
                    kahan_add(&k2, ((double)vdt[o] / dt) * n2);                                      \
                    kahan_add(&k3, 0.5 * gcoef * n2 * n2);                                           \
                }                                                                                    \
    out[0] = k0.s;                                                                                   \
    out[1] = k1.s;                                                                                   \
    out[2] = k2.s;                                                                                   \
    out[3] = k3.s;

void oracle_observables_f64(const oracle_grid *g, const double *psi, const double *vdt, double dt, double gcoef,
                            const double *w, double *out)
{
    OBSERVABLES_BODY(double)
}

void oracle_observables_f32(const oracle_grid *g, const float *psi, const float *vdt, double dt, double gcoef,
                            const double *w, double *out)
{
    OBSERVABLES_BODY(float)
}

long oracle_imaginary_f64(const oracle_grid *g, double *psi, double *work, const double *vdt, double dt,
                          double gcoef, const double *w, double vol, long steps, double tol, double *mu_hist)
{
    const size_t n = (size_t)g->nx * g->ny * g->nz * g->slots * 2;
    double *cur = psi, *nxt = work;
    double mu_prev = 0.0;
    long conv = -1;
    for (long k = 0; k < steps; k++) {
        double s[4];
        oracle_observables_f64(g, cur, vdt, dt, gcoef, w, s);
        const double nn = vol * s[0];
        const double mu = vol * (s[1] + s[2]) / nn + 2.0 * vol * s[3] / (nn * nn);
        if (mu_hist) mu_hist[k] = mu;
        if (k > 0 && conv < 0 && fabs(mu - mu_prev) < tol) conv = k;
        mu_prev = mu;
        oracle_half_step_f64(g, cur, nxt, vdt, 1, 1.0 / sqrt(nn));
        double *t = cur;
        cur = nxt;
        nxt = t;
    }
    double s[4];
    oracle_observables_f64(g, cur, vdt, dt, gcoef, w, s);
    const double sig = 1.0 / sqrt(vol * s[0]);
    for (size_t i = 0; i < n; i++) cur[i] = sig * cur[i];
    if (cur != psi) memcpy(psi, cur, n * sizeof(double));
    return conv;
}
