// spectrum.cu -- fused CIC deconvolution + log-k shell binning over the
// half-complex spectrum (the GPU counterpart of powerspectrum.c:35-111).
//
// Work split: each warp takes a contiguous block of (i, j) rows of N/2+1
// modes (the row counter is carried incrementally).  A row is walked in
// pieces of 32*RP modes; each piece is loaded coalesced into the warp's shared
// buffer and then every lane takes a contiguous run of RP modes (RP odd, so the
// strided shared reads are bank-conflict free).  Along a row |k| grows with kz,
// so a lane's bins are non-decreasing: the lane keeps one FP32 running sum per
// spectrum pair and flushes it (shared FP32 atomic) only when the bin changes.
// Every 16 rows the touched bin range is promoted into the warp's FP64
// histogram.  At the end the CTA sums its warps in a fixed order and writes one
// FP64 partial histogram; k_bin_finalize sums the partials of all CTAs in a
// fixed order and normalises, so results do not depend on scheduling.
//
// Per mode (powerspectrum.c:55-91): bin = max{b : thr[b] <= |k|^2} with the
// integer thresholds built on the host from the reference's own bin
// expression, weight c = 1 on the kz = 0 and kz = N/2 planes, 2 elsewhere,
// (0,0,0) skipped; value = c * Re(F_a F_b*) * p^4 where p = (iw_x*iw_y)*iw_z is
// the float product of the per-axis inverse windows (fieldize.cpp:129-132) and
// p^4 = invwindow^2.  Counts and mean |k| per bin are pure geometry and come
// from the host tables.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace genpk {
namespace {

struct BinParams {
    const float2 *f[kMaxBinFields];
    const double *corner[kMaxBinFields];  // exact (N/2,N/2,N/2) value per field, or null
    int64_t corner_row;                   // row index i*N+j of that mode, -1 if none
    int pa[kMaxBinPairs], pb[kMaxBinPairs];
    int np;          // pairs actually reported (<= NP of the instantiation)
    int dims, hc, half;
    int nrbins;
    float bpu_half;  // 0.5 * binsperunit as float, for the first-guess bin
    int rp;          // modes per lane per piece (odd)
    int warps;       // warps per CTA
};

constexpr int kBinBuf = 288;  // 32 * max RP (9) float2 per field per warp
constexpr int kPromoteRows = 16;  // rows summed in FP32 before promotion to FP64

// fv[idx] for a runtime idx without spilling fv to local memory.
template <int NF>
__device__ __forceinline__ float2 pick(const float2 (&fv)[NF], int idx)
{
    float2 r = fv[0];
#pragma unroll
    for (int f = 1; f < NF; f++)
        if (idx == f)
            r = fv[f];
    return r;
}

__device__ __forceinline__ int kval_dev(int i, int dims)
{
    return i <= dims / 2 ? i : i - dims;
}

// Bin of |k|^2 = kk2 >= 1: float first guess, then exact integer fix-up.
__device__ __forceinline__ int bin_lookup(uint32_t kk2, const uint32_t *thr, int nrbins,
                                          float bpu_half)
{
    int b = (int)(bpu_half * __logf((float)kk2));
    b = max(0, min(nrbins - 1, b));
    while (b + 1 < nrbins && kk2 >= thr[b + 1])
        b++;
    while (b > 0 && kk2 < thr[b])
        b--;
    return b;
}

// Shared layout (bytes):
//   thr  [nrbins+1] u32 | iw [hc] f32 | per warp: whist [NP][nrbins] f64,
//   rhist [NP][nrbins] f32, buf [NF][kBinBuf] float2
template <int NF, int NP>
__global__ void __launch_bounds__(256)
    k_bin(BinParams p, const uint32_t *__restrict__ thr_g, const float *__restrict__ iw_g,
          double *__restrict__ partial)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int nrb = p.nrbins;
    uint32_t *thr = (uint32_t *)smem;
    float *iwz = (float *)(thr + nrb + 1);
    size_t off = sizeof(uint32_t) * (nrb + 1) + sizeof(float) * p.hc;
    off = (off + 15) & ~(size_t)15;
    const size_t per_warp = ((sizeof(double) * NP * nrb + sizeof(float) * NP * nrb + 15) & ~(size_t)15) +
                            sizeof(float2) * NF * kBinBuf;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *wbase = smem + off + per_warp * wid;
    double *whist = (double *)wbase;
    float *rhist = (float *)(whist + NP * nrb);
    float2 *buf = (float2 *)(wbase + ((sizeof(double) * NP * nrb + sizeof(float) * NP * nrb + 15) &
                                      ~(size_t)15));

    for (int i = threadIdx.x; i <= nrb; i += blockDim.x)
        thr[i] = thr_g[i];
    for (int i = threadIdx.x; i < p.hc; i += blockDim.x)
        iwz[i] = iw_g[i];
    for (int i = lane; i < NP * nrb; i += 32) {
        whist[i] = 0.0;
        rhist[i] = 0.f;
    }
    __syncthreads();

    // Each warp takes a contiguous block of rows; (i, j) advance incrementally.
    const int64_t nrows = (int64_t)p.dims * p.dims;
    const int64_t gw = (int64_t)blockIdx.x * p.warps + wid;
    const int64_t nw = (int64_t)gridDim.x * p.warps;
    const int64_t per = (nrows + nw - 1) / nw;
    const int64_t r_begin = min(nrows, gw * per), r_end = min(nrows, r_begin + per);
    const int rp = p.rp;
    const int piece = 32 * rp;
    int i = (int)(r_begin / p.dims), j = (int)(r_begin - (int64_t)i * p.dims);
    int bmin = nrb, bmax = -1;  // this lane's bins since the last FP64 promotion
    int rows_since = 0;
    for (int64_t r = r_begin; r < r_end; r++) {
        const int ki = kval_dev(i, p.dims), kj = kval_dev(j, p.dims);
        const uint32_t r2 = (uint32_t)(ki * ki + kj * kj);
        const float pxy = __ldg(iw_g + i) * __ldg(iw_g + j);
        const size_t rowoff = (size_t)r * p.hc;
        int cb = -1;
        float acc[NP];
#pragma unroll
        for (int q = 0; q < NP; q++)
            acc[q] = 0.f;
        for (int pb = 0; pb < p.hc; pb += piece) {
            __syncwarp();
            for (int t = 0; t < rp; t++) {
                const int m = pb + t * 32 + lane;
                if (m < p.hc) {
#pragma unroll
                    for (int f = 0; f < NF; f++)
                        buf[f * kBinBuf + t * 32 + lane] = __ldg(p.f[f] + rowoff + m);
                }
            }
            __syncwarp();
            for (int t = 0; t < rp; t++) {
                const int q = lane * rp + t;
                const int kz = pb + q;
                if (kz >= p.hc)
                    break;
                const uint32_t kk2 = r2 + (uint32_t)(kz * kz);
                if (kk2 == 0)
                    continue;
                int b;
                if (cb < 0) {
                    b = bin_lookup(kk2, thr, nrb, p.bpu_half);
                } else {
                    b = cb;
                    while (b + 1 < nrb && kk2 >= thr[b + 1])
                        b++;
                }
                if (b != cb) {
                    if (cb >= 0) {
#pragma unroll
                        for (int s = 0; s < NP; s++) {
                            atomicAdd(&rhist[s * nrb + cb], acc[s]);
                            acc[s] = 0.f;
                        }
                    }
                    cb = b;
                    bmin = min(bmin, b);
                    bmax = max(bmax, b);
                }
                const float pz = pxy * iwz[kz];
                const float p2 = pz * pz;
                const float v = (kz == 0 || kz == p.half) ? p2 * p2 : 2.f * (p2 * p2);
                float2 fv[NF];
#pragma unroll
                for (int f = 0; f < NF; f++)
                    fv[f] = buf[f * kBinBuf + q];
                if (r == p.corner_row && kz == p.half) {
                    // The last log-k bin holds this single mode; its exact value
                    // (an alternating sum computed by the deposit) replaces the
                    // FP32 transform's, whose rounding noise it cannot average.
#pragma unroll
                    for (int f = 0; f < NF; f++)
                        if (p.corner[f])
                            fv[f] = make_float2((float)*p.corner[f], 0.f);
                }
#pragma unroll
                for (int s = 0; s < NP; s++) {
                    const float2 a = pick<NF>(fv, p.pa[s]), c = pick<NF>(fv, p.pb[s]);
                    acc[s] = fmaf(v, fmaf(a.x, c.x, a.y * c.y), acc[s]);
                }
            }
        }
        if (cb >= 0) {
#pragma unroll
            for (int s = 0; s < NP; s++)
                atomicAdd(&rhist[s * nrb + cb], acc[s]);
        }
        if (++j == p.dims) {
            j = 0;
            i++;
        }
        // Every kPromoteRows rows (and at the end) promote the FP32 sums of the
        // touched bins into the warp's FP64 histogram.
        if (++rows_since == kPromoteRows || r + 1 == r_end) {
            rows_since = 0;
            const int lo = (int)__reduce_min_sync(0xffffffffu, (unsigned)bmin);
            const int hi = (int)__reduce_max_sync(0xffffffffu, (unsigned)(bmax + 1)) - 1;
            __syncwarp();
            for (int b = lo + lane; b <= hi; b += 32) {
#pragma unroll
                for (int s = 0; s < NP; s++) {
                    whist[s * nrb + b] += (double)rhist[s * nrb + b];
                    rhist[s * nrb + b] = 0.f;
                }
            }
            __syncwarp();
            bmin = nrb;
            bmax = -1;
        }
    }
    __syncthreads();
    // CTA reduction in warp order -> one partial histogram per CTA.
    for (int k = threadIdx.x; k < p.np * nrb; k += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < p.warps; w++) {
            const double *wh = (const double *)(smem + off + per_warp * w);
            s += wh[k];
        }
        partial[(size_t)blockIdx.x * p.np * nrb + k] = s;
    }
}

struct NormParams {
    double ma[kMaxBinPairs], mb[kMaxBinPairs];
};

// One block per (pair, bin): strided sums over the CTA partials, then a
// fixed-order tree, so the result does not depend on scheduling.
constexpr int kFinalizeThreads = 256;

__global__ void __launch_bounds__(kFinalizeThreads)
    k_bin_finalize(const double *__restrict__ partial, int ctas, int np, int nrbins,
                   const double *__restrict__ count, NormParams mn, double *__restrict__ power)
{
    __shared__ double sh[kFinalizeThreads];
    const int k = blockIdx.x;
    const int s = k / nrbins, b = k - s * nrbins;
    double part = 0.0;
    for (int c = threadIdx.x; c < ctas; c += blockDim.x)
        part += partial[(size_t)c * np * nrbins + k];
    sh[threadIdx.x] = part;
    __syncthreads();
    for (int w = kFinalizeThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0)
        return;
    const double acc = sh[0];
    const double cnt = count[b];
    double out = 0.0;
    if (cnt > 0.0) {
        out = acc / (mn.ma[s] * mn.mb[s]);
        out /= cnt;
    }
    power[k] = out;
}

size_t bin_smem(int nrbins, int hc, int np, int nf, int warps)
{
    size_t off = sizeof(uint32_t) * (nrbins + 1) + sizeof(float) * hc;
    off = (off + 15) & ~(size_t)15;
    const size_t per_warp = ((sizeof(double) * np * nrbins + sizeof(float) * np * nrbins + 15) &
                             ~(size_t)15) +
                            sizeof(float2) * nf * kBinBuf;
    return off + per_warp * warps;
}

// Instantiated (fields, pairs) shapes; a request is rounded up to the first
// shape that holds it and padded with dummy pairs whose sums are dropped.
struct Shape {
    int nf, np;
};
constexpr Shape kShapes[] = {{1, 1}, {2, 1}, {2, 3}, {3, 6}, {4, 10}};

Shape pick_shape(int nf, int np)
{
    for (const Shape &s : kShapes)
        if (s.nf >= nf && s.np >= np)
            return s;
    return {0, 0};
}

}  // namespace

int bin_ctas(const GridGeom &g, int nrbins, int npairs, int nfields, int num_sms, int *warps,
             size_t *smem)
{
    const Shape s = pick_shape(nfields, npairs);
    if (s.nf == 0)
        return 0;
    int w = 8;
    while (w > 1 && bin_smem(nrbins, g.hc, s.np, s.nf, w) > 200 * 1024)
        w /= 2;
    const size_t sm = bin_smem(nrbins, g.hc, s.np, s.nf, w);
    if (sm > 220 * 1024)
        return 0;
    *warps = w;
    *smem = sm;
    const int per_sm = std::max(1, std::min(2048 / (32 * w), (int)((220 * 1024) / sm)));
    const int64_t rows = (int64_t)g.dims * g.dims;
    const int64_t want = (rows + w - 1) / w;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms * per_sm, want));
}

cudaError_t bin_spectra(const GridGeom &g, const BinTables &t, const BinDevice &d,
                        const BinLaunch &l, double *partial, double *out_power, int ctas,
                        int warps, size_t smem, cudaStream_t stream, int64_t *launches)
{
    const Shape s = pick_shape(l.nfields, l.npairs);
    BinParams p;
    for (int f = 0; f < kMaxBinFields; f++) {
        p.f[f] = l.fields[f < l.nfields ? f : 0];
        p.corner[f] = l.corner[f < l.nfields ? f : 0];
    }
    p.corner_row = (g.dims % 2 == 0) ? (int64_t)g.half * g.dims + g.half : -1;
    for (int q = 0; q < kMaxBinPairs; q++) {
        const int src = q < l.npairs ? q : 0;
        p.pa[q] = l.pairs[src].a;
        p.pb[q] = l.pairs[src].b;
    }
    p.np = l.npairs;
    p.dims = g.dims;
    p.hc = g.hc;
    p.half = g.half;
    p.nrbins = t.nrbins;
    p.bpu_half = (float)(0.5 * t.binsperunit);
    p.rp = g.hc <= 32 ? 1 : g.hc <= 96 ? 3 : g.hc <= 160 ? 5 : 9;
    p.warps = warps;
    cudaError_t err;
#define GENPK_BIN_LAUNCH(NF, NP)                                                              \
    do {                                                                                      \
        auto kern = k_bin<NF, NP>;                                                            \
        if ((err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                        (int)smem)) != cudaSuccess)                           \
            return err;                                                                       \
        kern<<<ctas, 32 * warps, smem, stream>>>(p, d.thr, d.iw, partial);                    \
    } while (0)
    if (s.nf == 1)
        GENPK_BIN_LAUNCH(1, 1);
    else if (s.nf == 2 && s.np == 1)
        GENPK_BIN_LAUNCH(2, 1);
    else if (s.nf == 2)
        GENPK_BIN_LAUNCH(2, 3);
    else if (s.nf == 3)
        GENPK_BIN_LAUNCH(3, 6);
    else
        GENPK_BIN_LAUNCH(4, 10);
#undef GENPK_BIN_LAUNCH
    (*launches)++;
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    NormParams mn;
    for (int q = 0; q < kMaxBinPairs; q++) {
        mn.ma[q] = q < l.npairs ? l.pairs[q].mass_a : 1.0;
        mn.mb[q] = q < l.npairs ? l.pairs[q].mass_b : 1.0;
    }
    const int k = l.npairs * t.nrbins;
    k_bin_finalize<<<k, kFinalizeThreads, 0, stream>>>(partial, ctas, l.npairs, t.nrbins, d.count,
                                                        mn, out_power);
    (*launches)++;
    return cudaGetLastError();
}

}  // namespace genpk
