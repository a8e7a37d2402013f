// tables.cpp -- host-side bin and window tables, evaluated with the reference's
// own expressions so that bin edges and window factors round identically.
//
// Built with the reference's floating-point flags (-O2 -ffast-math,
// Makefile:30-37): the bin index floor(binsperunit*log(kk)) of
// powerspectrum.c:38,66,84 is sensitive to the last ulp of log, and mode counts
// must match the reference bit for bit.
//
//   ref_onedinvwindow   fieldize.cpp:117-121
//   ref_invwindow       fieldize.cpp:125-133
//   bin index           powerspectrum.c:38 (binsperunit), :66/:84 (floor(b*log(kk)))
//   counts / keffs      powerspectrum.c:55-91 weights, :102-108 normalisation
#include <math.h>

#include <algorithm>
#include <cstdio>

#include "internal.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace genpk {

double ref_onedinvwindow(int64_t k, int64_t n)
{
    return k ? M_PI * k / (n * sin(M_PI * k / (float)n)) : 1.0;
}

double ref_invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n)
{
    if (n == 0)
        return 0;
    const float iwx = ref_onedinvwindow(kx, n);
    const float iwy = ref_onedinvwindow(ky, n);
    const float iwz = ref_onedinvwindow(kz, n);
    const float p = iwx * iwy * iwz;
    return (double)p * (double)p;
}

namespace {

int64_t kval_host(int64_t i, int64_t dims)
{
    return i <= dims / 2 ? i : i - dims;
}

// floor(binsperunit * log(sqrt(kk2))), the reference expression.
int64_t ref_bin(int64_t kk2, double binsperunit)
{
    const double kk = sqrt((double)kk2);
    return (int64_t)floor(binsperunit * log(kk));
}

}  // namespace

int64_t table_kk2max(int64_t dims)
{
    const int64_t half = dims / 2;
    return 3 * half * half;
}

int64_t table_r2max(int64_t dims)
{
    const int64_t half = dims / 2;
    return 2 * half * half;
}

bool build_bin_tables_into(int64_t dims, int nrbins, const TableSpans &o, double *binsperunit_out,
                           const char **why)
{
    const double binsperunit = (nrbins - 1) / log(sqrt(3) * dims / 2.0);
    *binsperunit_out = binsperunit;
    const int64_t half = dims / 2;
    const int64_t r2max = table_r2max(dims);
    const int64_t kk2max = table_kk2max(dims);
    if (kk2max > 0x7fffffffLL) {
        *why = "grid too large for 32-bit |k|^2";
        return false;
    }
    // Bin of every integer |k|^2, and the thresholds thr[b] = min{kk2 : bin >= b}.
    o.lut[0] = -1;
    for (int b = 0; b <= nrbins; b++)
        o.thr[b] = 0xffffffffu;
    int64_t prev = -1;
    for (int64_t kk2 = 1; kk2 <= kk2max; kk2++) {
        const int64_t b = ref_bin(kk2, binsperunit);
        if (b < 0 || b >= nrbins) {
            *why = "bin index out of range";
            return false;
        }
        if (b < prev) {
            *why = "bin index not monotone in |k|^2";
            return false;
        }
        for (int64_t q = prev + 1; q <= b; q++)
            o.thr[q] = (uint32_t)kk2;
        prev = b;
        o.lut[kk2] = (int32_t)b;
    }
    for (int64_t i = 0; i < dims; i++)
        o.iw[i] = (float)ref_onedinvwindow(kval_host(i, dims), dims);

    // Weighted mode counts and mean |k| per bin.  The (i, j) pairs are grouped by
    // r2 = ki^2 + kj^2 first, so the loop is over distinct r2 values times kz.
    for (int64_t r2 = 0; r2 <= r2max; r2++)
        o.cnt2[r2] = 0;
    for (int64_t i = 0; i < dims; i++) {
        const int64_t ki = kval_host(i, dims);
        for (int64_t j = 0; j < dims; j++) {
            const int64_t kj = kval_host(j, dims);
            o.cnt2[ki * ki + kj * kj]++;
        }
    }
    for (int b = 0; b < nrbins; b++) {
        o.count[b] = 0;
        o.keffs[b] = 0.0;
    }
    for (int64_t r2 = 0; r2 <= r2max; r2++) {
        const int64_t c2 = o.cnt2[r2];
        if (!c2)
            continue;
        for (int64_t kz = 0; kz <= half; kz++) {
            const int64_t kk2 = r2 + kz * kz;
            if (kk2 == 0)
                continue;
            const int64_t w = (kz == 0 || kz == half) ? 1 : 2;
            const int32_t b = o.lut[kk2];
            o.count[b] += w * c2;
            o.keffs[b] += (double)(w * c2) * sqrt((double)kk2);
        }
    }
    for (int b = 0; b < nrbins; b++)
        if (o.count[b])
            o.keffs[b] /= (double)o.count[b];
    return true;
}

bool build_bin_tables(int64_t dims, int nrbins, BinTables *t, std::string *err)
{
    t->dims = dims;
    t->nrbins = nrbins;
    t->kk2max = table_kk2max(dims);
    if (t->kk2max > 0x7fffffffLL) {
        *err = "grid too large for 32-bit |k|^2";
        return false;
    }
    t->lut.assign((size_t)t->kk2max + 1, -1);
    t->thr.assign((size_t)nrbins + 1, 0xffffffffu);
    t->iw.assign((size_t)dims, 0.f);
    t->count.assign((size_t)nrbins, 0);
    t->keffs.assign((size_t)nrbins, 0.0);
    std::vector<int64_t> cnt2((size_t)table_r2max(dims) + 1, 0);
    TableSpans o{t->thr.data(), t->iw.data(), t->count.data(), t->keffs.data(), t->lut.data(),
                 cnt2.data()};
    const char *why = nullptr;
    if (!build_bin_tables_into(dims, nrbins, o, &t->binsperunit, &why)) {
        *err = why;
        return false;
    }
    return true;
}

}  // namespace genpk
