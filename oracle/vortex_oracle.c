/*
 * vortex_oracle.c - CPU oracle for the axisymmetric vortex relaxation.  TEST
 * INFRASTRUCTURE ONLY: loaded by tests/ and bench.py's CPU-baseline leg as the
 * checker; never part of the shipped library.
 *
 * A plain-C restatement of markus-kivioja/vaikkari,
 * koodit/GrossPitaevskii/VortexState.cpp:
 *   - setRange / setDimensions initial state:  :12-47
 *   - initialize (bilinear resampling):        :98-107 with getFunction :213-238
 *   - iterateSolution (Gauss-Seidel sweep, norm, mu, rescale, sign):  :109-185
 *   - searchFunctionMax / searchMinR / searchMaxR / searchMaxZ:       :240-280
 * with the potential potentialRZ of GPUGrossPitaevskii_BCC.cu:28-31
 * (0.5 * (r^2 + RATIO^2 z^2), RATIO = 0.1 there).  Every expression keeps the
 * reference's operation order; compiled with -ffp-contract=off.
 *
 * Two summation orders for the per-iteration sums (diff, prob, prob2) and the
 * final sign test:
 *   order 0: one running sum over all points in sweep order (the reference);
 *   order 1: per row, one running sum per chunk of `chunk` consecutive
 *            columns, chunk sums added in column order to a row sum; row sums
 *            added in groups of 16 consecutive rows, group sums in order (the
 *            GPU kernels' order).
 * The sweep itself is identical in both.
 */
#include <math.h>
#include <stddef.h>

static const double kPI = 3.1415926535897932385;   /* jukan_koodit/Types/Types.hpp:20-21 */
static const double kPIx2 = 6.2831853071795864770;

/* setDimensions (VortexState.cpp:12-40): the initial state. */
void oracle_vortex_initial(unsigned rsize, double rstep, double rplug, unsigned zsize, double zstep, double *f)
{
    double prob = 0.0;
    size_t ii = 0;
    for (unsigned i = 0; i < rsize; i++) {
        const double fr = 1.0 - cos(i * kPIx2 / (double)rsize);
        const double r = rplug + i * rstep;
        unsigned times = 1;
        for (unsigned j = 0; j < zsize; j++, ii++) {
            f[ii] = (1.0 + cos(j * kPI / (double)zsize)) * fr;
            prob += times * f[ii] * f[ii] * r;
            times = 2;
        }
    }
    prob *= kPIx2 * rstep * zstep;
    const double scale = 1.0 / sqrt(prob);
    for (ii = 0; ii < (size_t)rsize * zsize; ii++) f[ii] *= scale;
}

/* getFunction (VortexState.cpp:213-238). */
double oracle_vortex_function(const double *f, unsigned rsize, unsigned zsize, double rplug, double rstep,
                              double zstep, double r, double z)
{
    const double rr = (r - rplug) / rstep;
    if (rr < 0.0) return 0.0;
    const unsigned ir = (unsigned)rr;
    if (ir >= rsize) return 0.0;
    const double dr = rr - (double)ir;
    const double zz = fabs(z) / zstep;
    const unsigned iz = (unsigned)zz;
    if (iz >= zsize) return 0.0;
    const double dz = zz - (double)iz;
    const size_t ii = (size_t)ir * zsize + iz;
    const double fiir = (ir + 1 < rsize ? f[ii + zsize] : 0.0);
    const double fiiz = (iz + 1 < zsize ? f[ii + 1] : 0.0);
    const double fiirz = (ir + 1 < rsize && iz + 1 < zsize ? f[ii + zsize + 1] : 0.0);
    return (1.0 - dz) * ((1.0 - dr) * f[ii] + dr * fiir) + dz * ((1.0 - dr) * fiiz + dr * fiirz);
}

/* initialize (VortexState.cpp:98-107): resample src onto the grid of dst. */
void oracle_vortex_resample(const double *src, unsigned rs, unsigned zs, double rplug_s, double rstep_s,
                            double zstep_s, double *dst, unsigned rd, unsigned zd, double rplug_d, double rstep_d,
                            double zstep_d)
{
    size_t ii = 0;
    for (unsigned i = 0; i < rd; i++) {
        const double r = rplug_d + i * rstep_d;
        for (unsigned j = 0; j < zd; j++) dst[ii++] = oracle_vortex_function(src, rs, zs, rplug_s, rstep_s, zstep_s,
                                                                             r, j * zstep_d);
    }
}

typedef struct {
    int order, chunk, row_group;
    double total, group, row, part;
    unsigned j_in_chunk, rows_in_group;
} summer;

static void sum_begin(summer *s, int order, int chunk)
{
    s->order = order;
    s->chunk = chunk;
    s->row_group = 16;
    s->total = s->group = s->row = s->part = 0.0;
    s->rows_in_group = 0;
}
static void sum_row_begin(summer *s)
{
    s->row = s->part = 0.0;
    s->j_in_chunk = 0;
}
static void sum_add(summer *s, double x)
{
    if (s->order == 0) {
        s->total += x;
        return;
    }
    s->part += x;
    if (++s->j_in_chunk == (unsigned)s->chunk) {
        s->row += s->part;
        s->part = 0.0;
        s->j_in_chunk = 0;
    }
}
static void sum_row_end(summer *s)
{
    if (s->order == 0) return;
    if (s->j_in_chunk) s->row += s->part;
    s->group += s->row;
    if (++s->rows_in_group == (unsigned)s->row_group) {
        s->total += s->group;
        s->group = 0.0;
        s->rows_in_group = 0;
    }
}

static double sum_total(summer *s)
{
    if (s->order == 1 && s->rows_in_group) {
        s->total += s->group;
        s->group = 0.0;
        s->rows_in_group = 0;
    }
    return s->total;
}

/* iterateSolution (VortexState.cpp:109-185).  Returns the iterations run
 * (k + 1 at the break, else maxiters); *mu is read and updated; *last_diff
 * receives the last sweep's diff. */
long oracle_vortex_iterate(double *f, unsigned rsize, unsigned zsize, double rplug, double rstep, double zstep,
                           unsigned kappa, double g, double ratio, double *mu, long maxiters, double eps, int order,
                           int chunk, double *last_diff)
{
    const double PIx2drdz = kPIx2 * rstep * zstep;
    const double kk = 0.5 * (double)(kappa * kappa);
    const double laplr = 0.5 / (rstep * rstep);
    const double laplz = (zsize > 1 ? 0.5 / (zstep * zstep) : 0.0);
    const size_t n = (size_t)rsize * zsize;
    long k;
    double diffv = 0.0;
    for (unsigned j = 0; j < zsize; j++) f[j] = 0.0;
    for (k = 0; k < maxiters; k++) {
        summer diff;
        sum_begin(&diff, order, chunk);
        size_t ii = zsize;
        for (unsigned i = 1; i < rsize; i++) {
            const double r = rplug + i * rstep;
            const double lapl = kk / (r * r) + 2.0 * (laplr + laplz);
            const double gradr = 0.25 / (r * rstep);
            double dv = PIx2drdz * r;
            sum_row_begin(&diff);
            for (unsigned j = 0; j < zsize; j++, ii++) {
                const double z = j * zstep;
                const double pot = 0.5 * (r * r + ratio * ratio * z * z) + g * f[ii] * f[ii];
                const double fiir = (i + 1 < rsize ? f[ii + zsize] : 0.0);
                const double frii = f[ii - zsize];
                const double fiiz = (j + 1 < zsize ? f[ii + 1] : 0.0);
                const double fzii = (j > 0 ? f[ii - 1] : fiiz);
                double dfii = f[ii];
                f[ii] = (gradr * (frii - fiir) - laplr * (frii + fiir) - laplz * (fzii + fiiz)) / (*mu - lapl - pot);
                dfii -= f[ii];
                sum_add(&diff, dfii * dfii * dv);
                if (j == 0) dv *= 2.0;
            }
            sum_row_end(&diff);
        }
        summer prob, prob2;
        sum_begin(&prob, order, chunk);
        sum_begin(&prob2, order, chunk);
        ii = zsize;
        for (unsigned i = 1; i < rsize; i++) {
            const double r = rplug + i * rstep;
            const double lapl = kk / (r * r) + 2.0 * (laplr + laplz);
            const double gradr = 0.25 / (r * rstep);
            double dv = PIx2drdz * r;
            sum_row_begin(&prob);
            sum_row_begin(&prob2);
            for (unsigned j = 0; j < zsize; j++, ii++) {
                const double z = j * zstep;
                const double pot = 0.5 * (r * r + ratio * ratio * z * z) + g * f[ii] * f[ii];
                const double fiir = (i + 1 < rsize ? f[ii + zsize] : 0.0);
                const double frii = f[ii - zsize];
                const double fiiz = (j + 1 < zsize ? f[ii + 1] : 0.0);
                const double fzii = (j > 0 ? f[ii - 1] : fiiz);
                sum_add(&prob, f[ii] * f[ii] * dv);
                sum_add(&prob2, ((pot + lapl) * f[ii] + gradr * (frii - fiir) - laplr * (frii + fiir) -
                                 laplz * (fzii + fiiz)) * f[ii] * dv);
                if (j == 0) dv *= 2.0;
            }
            sum_row_end(&prob);
            sum_row_end(&prob2);
        }
        const double tp = sum_total(&prob), tp2 = sum_total(&prob2);
        *mu = tp2 / tp;
        const double scale = 1.0 / sqrt(tp);
        for (ii = zsize; ii < n; ii++) f[ii] *= scale;
        diffv = sum_total(&diff);
        if (diffv < eps) {
            k++;
            break;
        }
    }
    /* make f non-negative */
    summer s;
    sum_begin(&s, order, chunk);
    size_t ii = zsize;
    for (unsigned i = 1; i < rsize; i++) {
        sum_row_begin(&s);
        for (unsigned j = 0; j < zsize; j++, ii++) sum_add(&s, f[ii]);
        sum_row_end(&s);
    }
    if (sum_total(&s) < 0.0)
        for (ii = zsize; ii < n; ii++) f[ii] = -f[ii];
    if (last_diff) *last_diff = diffv;
    return k;
}

/* searchFunctionMax, searchMinR, searchMaxR, searchMaxZ (VortexState.cpp:240-280). */
double oracle_vortex_function_max(const double *f, size_t n)
{
    double m = 0.0;
    for (size_t ii = 0; ii < n; ii++)
        if (f[ii] > m) m = f[ii];
    return m;
}

double oracle_vortex_min_r(const double *f, unsigned rsize, unsigned zsize, double rplug, double rstep, double eps)
{
    for (size_t ii = 0; ii < (size_t)rsize * zsize; ii++)
        if (f[ii] > eps) return rplug + (double)(unsigned)(ii / zsize) * rstep;
    return 1e30;
}
