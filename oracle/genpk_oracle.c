/*
 * genpk_oracle.c -- CPU restatement of GenPK's power-spectrum hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * path in genpk_gb300/csrc.  It is built by oracle/Makefile and loaded only by
 * tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and the
 * --impl reference arm).  Nothing in the product library links or calls it.
 *
 * Everything here is computed in FP64, as in the reference (GENFLOAT is
 * double, gen-pk.h:31).  The FFT between deposit and binning is not here: the
 * Python side (oracle/oracle.py) uses numpy's FP64 pocketfft, which follows
 * FFTW's r2c convention (unnormalised, e^{-ikx}).
 *
 * It is compiled with the reference's flags (-O2 -ffast-math -fopenmp,
 * Makefile:30-37) so that the bin index expression floor(b*log(kk)) rounds the
 * same way the reference build does.
 *
 * Functions and the reference code they restate:
 *   oracle_fieldize      fieldize.cpp:46-113   CIC deposit, += into padded grid
 *   oracle_onedinvwindow fieldize.cpp:117-121  1-D inverse CIC window
 *   oracle_invwindow     fieldize.cpp:125-133  3-D inverse window, per-axis float
 *   oracle_powerspectrum powerspectrum.c:35-111 deconvolved |F|^2 log-k binning
 *   oracle_cic_gather    (no reference counterpart) exact transpose of
 *                        oracle_fieldize, used for the FP64 reference gradient
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Particles handled per batch between two scatter phases.  The reference
 * buffers 64 particles per thread and serialises the scatter in an OpenMP
 * critical section (fieldize.cpp:24,53-111); the same structure is kept here so
 * that the CPU timing of this port is representative of the reference. */
#define ORACLE_BATCH 64

/* Wrap a cell index into [0, n) the way fieldize.cpp:70-75 does. */
static inline int64_t wrap_cell(int64_t c, int64_t n)
{
    int64_t r = c % n;
    return r < 0 ? r + n : r;
}

/* CIC weights and cell offsets of one particle (fieldize.cpp:60-92).
 * Corner bit 0 selects x+1, bit 1 y+1, bit 2 z+1. */
static inline void cic_corners(const float *p, double units, int64_t dims,
                               size_t row, size_t plane, double m,
                               double w[8], size_t idx[8])
{
    double d[3], t[3];
    int64_t lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        double x = (double)p[a] * units;
        int64_t f = (int64_t)floor(x);
        d[a] = x - (double)f;
        t[a] = 1.0 - d[a];
        hi[a] = wrap_cell(f + 1, dims);
        lo[a] = wrap_cell(f, dims);
    }
    for (int c = 0; c < 8; c++) {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        w[c] = m * (bx ? d[0] : t[0]) * (by ? d[1] : t[1]) * (bz ? d[2] : t[2]);
        idx[c] = plane * (size_t)(bx ? hi[0] : lo[0]) +
                 row * (size_t)(by ? hi[1] : lo[1]) + (size_t)(bz ? hi[2] : lo[2]);
    }
}

/* fieldize.cpp:46-113.  out is the padded grid: row length fdims =
 * 2*(dims/2+extra), so with extra=1 it is the FFTW in-place r2c layout. */
int oracle_fieldize(double boxsize, int dims, double *out, int64_t n,
                    const float *pos, const float *masses, double mass, int extra)
{
    const size_t row = 2 * (size_t)(dims / 2 + extra);
    const size_t plane = row * (size_t)dims;
    const double units = dims / boxsize;
#pragma omp parallel for schedule(static)
    for (int64_t b0 = 0; b0 < n; b0 += ORACLE_BATCH) {
        double w[ORACLE_BATCH][8];
        size_t idx[ORACLE_BATCH][8];
        const int64_t nb = (n - b0 < ORACLE_BATCH) ? n - b0 : ORACLE_BATCH;
        for (int64_t q = 0; q < nb; q++) {
            const int64_t p = b0 + q;
            const double m = masses ? (double)masses[p] : mass;
            cic_corners(pos + 3 * p, units, dims, row, plane, m, w[q], idx[q]);
        }
#pragma omp critical(oracle_scatter)
        {
            for (int64_t q = 0; q < nb; q++)
                for (int c = 0; c < 8; c++)
                    out[idx[q][c]] += w[q][c];
        }
    }
    return 0;
}

/* fieldize.cpp:117-121: pi k / (n sin(pi k / n)), 1 at k = 0.  The inner
 * division is by (float)n, as in the reference. */
double oracle_onedinvwindow(int64_t k, int64_t n)
{
    if (k == 0)
        return 1.0;
    return M_PI * (double)k / ((double)n * sin(M_PI * (double)k / (float)n));
}

/* fieldize.cpp:125-133: each axis factor is stored as float before the product,
 * and the float product is squared in double. */
double oracle_invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n)
{
    if (n == 0)
        return 0.0;
    const float ax = (float)oracle_onedinvwindow(kx, n);
    const float ay = (float)oracle_onedinvwindow(ky, n);
    const float az = (float)oracle_onedinvwindow(kz, n);
    const float prod = ax * ay * az;
    return (double)prod * (double)prod;
}

/* Signed wavenumber of storage index i (powerspectrum.c:33, KVAL). */
static inline int64_t kval(int64_t i, int64_t dims)
{
    return i <= dims / 2 ? i : i - dims;
}

/* Bin index of a mode with integer |k|^2 = kk2 (powerspectrum.c:38,66,84). */
static inline int64_t bin_of(double kk2, double binsperunit)
{
    const double kk = sqrt(kk2);
    return (int64_t)floor(binsperunit * log(kk));
}

/* Bin index of integer |k|^2, exported so tests can compare the GPU library's
 * bin table against exactly this expression. */
int64_t oracle_bin_of(int64_t kk2, int64_t dims, int nrbins)
{
    const double binsperunit = (nrbins - 1) / log(sqrt(3) * dims / 2.0);
    return bin_of((double)kk2, binsperunit);
}

/* One mode's contribution: weight * Re(F1 F2*) * invwindow^2
 * (powerspectrum.c:68,77,86).  f1/f2 point at interleaved (re, im). */
static inline double mode_power(const double *f1, const double *f2, int64_t m,
                                double win)
{
    return (f1[2 * m] * f2[2 * m] + f1[2 * m + 1] * f2[2 * m + 1]) * win * win;
}

/* powerspectrum.c:35-111.  f1, f2: the half-complex spectrum, dims*dims*(dims/2+1)
 * complex values stored as interleaved doubles.  Per-thread private histograms
 * merged in a critical section, as in the reference. */
int oracle_powerspectrum(int64_t dims, const double *f1, const double *f2,
                         int nrbins, double *power, int *count, double *keffs,
                         double m1, double m2)
{
    const double binsperunit = (nrbins - 1) / log(sqrt(3) * dims / 2.0);
    const int64_t half = dims / 2;
    memset(power, 0, sizeof(double) * nrbins);
    memset(count, 0, sizeof(int) * nrbins);
    memset(keffs, 0, sizeof(double) * nrbins);
#pragma omp parallel
    {
        double *pp = calloc((size_t)nrbins, sizeof(double));
        double *kp = calloc((size_t)nrbins, sizeof(double));
        int *cp = calloc((size_t)nrbins, sizeof(int));
#pragma omp for schedule(static) nowait
        for (int64_t i = 0; i < dims; i++) {
            const int64_t ki = kval(i, dims);
            for (int64_t j = 0; j < dims; j++) {
                const int64_t kj = kval(j, dims);
                const int64_t rowbase = (i * dims + j) * (half + 1);
                const int64_t r2 = ki * ki + kj * kj;
                /* kz = 0 plane, weight 1, the (0,0,0) mode skipped. */
                if (r2 > 0) {
                    const int64_t b = bin_of((double)r2, binsperunit);
                    pp[b] += mode_power(f1, f2, rowbase, oracle_invwindow(ki, kj, 0, dims));
                    kp[b] += sqrt((double)r2);
                    cp[b] += 1;
                }
                /* kz = dims/2 plane, weight 1. */
                {
                    const int64_t kz = kval(half, dims);
                    const int64_t kk2 = r2 + kz * kz;
                    const int64_t b = bin_of((double)kk2, binsperunit);
                    pp[b] += mode_power(f1, f2, rowbase + half, oracle_invwindow(ki, kj, kz, dims));
                    kp[b] += sqrt((double)kk2);
                    cp[b] += 1;
                }
                /* 0 < kz < dims/2, weight 2 for the conjugate partner. */
                for (int64_t k = 1; k < half; k++) {
                    const int64_t kk2 = r2 + k * k;
                    const int64_t b = bin_of((double)kk2, binsperunit);
                    pp[b] += 2.0 * mode_power(f1, f2, rowbase + k, oracle_invwindow(ki, kj, k, dims));
                    kp[b] += 2.0 * sqrt((double)kk2);
                    cp[b] += 2;
                }
            }
        }
#pragma omp critical(oracle_merge)
        for (int b = 0; b < nrbins; b++) {
            power[b] += pp[b];
            count[b] += cp[b];
            keffs[b] += kp[b];
        }
        free(pp);
        free(kp);
        free(cp);
    }
    for (int b = 0; b < nrbins; b++) {
        if (count[b]) {
            power[b] /= m1 * m2;
            power[b] /= count[b];
            keffs[b] /= count[b];
        }
    }
    return 0;
}

/* Transpose of oracle_fieldize: for each particle, the CIC-weighted gather of
 * a padded real grid g (the gradient of a loss with respect to the density)
 * and its derivative with respect to the particle's position.
 *   gmass[p]   = sum_c w_c g(corner_c) / m_p  (gradient w.r.t. the mass)
 *   gpos[p][a] = m_p * units * sum_c (+-1 on axis a) prod_{e!=a} w_e g(corner_c)
 * No reference counterpart: the reference computes no derivative. */
int oracle_cic_gather(double boxsize, int dims, const double *g, int64_t n,
                      const float *pos, const float *masses, double mass,
                      double *gpos, double *gmass)
{
    const size_t row = 2 * (size_t)(dims / 2 + 1);
    const size_t plane = row * (size_t)dims;
    const double units = dims / boxsize;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; p++) {
        double d[3], t[3];
        int64_t lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            const double x = (double)pos[3 * p + a] * units;
            const int64_t f = (int64_t)floor(x);
            d[a] = x - (double)f;
            t[a] = 1.0 - d[a];
            hi[a] = wrap_cell(f + 1, dims);
            lo[a] = wrap_cell(f, dims);
        }
        const double m = masses ? (double)masses[p] : mass;
        double sw = 0.0, dg[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 8; c++) {
            const int b[3] = {c & 1, (c >> 1) & 1, (c >> 2) & 1};
            const double v = g[plane * (size_t)(b[0] ? hi[0] : lo[0]) +
                               row * (size_t)(b[1] ? hi[1] : lo[1]) +
                               (size_t)(b[2] ? hi[2] : lo[2])];
            double f3[3];
            for (int a = 0; a < 3; a++)
                f3[a] = b[a] ? d[a] : t[a];
            sw += f3[0] * f3[1] * f3[2] * v;
            for (int a = 0; a < 3; a++) {
                const double s = b[a] ? 1.0 : -1.0;
                dg[a] += s * f3[(a + 1) % 3] * f3[(a + 2) % 3] * v;
            }
        }
        gmass[p] = sw;
        for (int a = 0; a < 3; a++)
            gpos[3 * p + a] = m * units * dg[a];
    }
    return 0;
}

/* Number of OpenMP threads the port runs with (reported as cpu_baseline.cores). */
int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
