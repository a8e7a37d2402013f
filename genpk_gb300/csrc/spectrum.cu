// spectrum.cu -- fused CIC deconvolution + log-k shell binning over the
// half-complex spectrum (the GPU counterpart of powerspectrum.c:35-111).
//
// Work split: each warp takes a contiguous block of (i, j) rows of N/2+1
// modes, walked in pieces of 32*RP modes with the next piece's loads in
// flight.  Every lane bins a contiguous run of RP modes; bins only grow along a
// run, so a lane keeps one FP32 running sum per spectrum pair and compares
// |k|^2 with the next threshold held in a register.  The lanes' open sums are
// combined at the end of a piece by a segmented warp scan over their bins (no
// atomics); a bin completed inside a run (only where bins are narrower than a
// run) goes to the warp's FP32 histogram with a shared atomic.  Every 16 rows
// the touched bins are promoted into the warp's FP64 histogram.  At the end
// the CTA sums its warps in a fixed order and writes one FP64 partial
// histogram; k_bin_finalize sums the partials of all CTAs in a fixed order and
// normalises, so results do not depend on scheduling.
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
    int np;          // pair sums per CTA partial: the instantiation's pair count
    int dims, hc, half;
    int nrbins;
    float bpu_half;  // 0.5 * binsperunit as float, for the first-guess bin
    int rp;          // modes per lane per piece (odd)
    int warps;       // warps per CTA
};

constexpr int kPromoteRows = 16;  // rows summed in FP32 before promotion to FP64

// Pairs an instantiation sums, with compile-time field indices: the single
// cross pair (0, 1) (CROSS1), or every pair a <= b of NF fields in the order
// (0,0), (0,1), ..., (0,NF-1), (1,1), ... (Re F_a F_b* is symmetric).
template <int NF, bool CROSS1>
struct PairSet {
    static constexpr int NP = CROSS1 ? 1 : NF * (NF + 1) / 2;
};

__host__ __device__ constexpr int pair_slot(int nf, int a, int b)
{
    return a * nf - a * (a - 1) / 2 + (b - a);
}

template <int NF, bool CROSS1>
__device__ __forceinline__ void add_pairs(const float2 (&fv)[NF], float w,
                                          float (&acc)[PairSet<NF, CROSS1>::NP])
{
    if (CROSS1) {
        acc[0] = fmaf(w, fmaf(fv[0].x, fv[NF - 1].x, fv[0].y * fv[NF - 1].y), acc[0]);
    } else {
#pragma unroll
        for (int a = 0; a < NF; a++)
#pragma unroll
            for (int b = a; b < NF; b++)
                acc[pair_slot(NF, a, b)] =
                    fmaf(w, fmaf(fv[a].x, fv[b].x, fv[a].y * fv[b].y), acc[pair_slot(NF, a, b)]);
    }
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

// Shared layout (bytes, each block 16-byte aligned):
//   thr [nrbins+1] u32 | izc [hc] float2 {iw(kz), mode weight 1 or 2} |
//   per warp: whist [NP][nrbins] f64, rhist [NP][nrbins] f32, buf [NF][32*RP] float2
struct BinLayout {
    size_t izc, warps, whist, rhist, buf, per_warp;
};

__host__ __device__ inline size_t align16(size_t v)
{
    return (v + 15) & ~(size_t)15;
}

__host__ __device__ inline BinLayout bin_layout(int nrbins, int hc, int np, int nf, int rp)
{
    BinLayout L;
    L.izc = align16(sizeof(uint32_t) * (nrbins + 1));
    L.warps = L.izc + align16(sizeof(float2) * hc);
    L.whist = 0;
    L.rhist = align16(sizeof(double) * np * nrbins);
    L.buf = L.rhist + align16(sizeof(float) * np * nrbins);
    L.per_warp = L.buf + sizeof(float2) * nf * 32 * rp;
    return L;
}

constexpr int kMaxRP = 9;

// One piece of a row: 32*RP consecutive modes from kz = pb, field values into
// registers (coalesced loads; zero past the row's end).
template <int NF>
__device__ __forceinline__ void load_piece(const BinParams &p, int64_t r, int pb, int lane,
                                           float2 (&v)[NF][kMaxRP])
{
    const size_t rowoff = (size_t)r * p.hc;
#pragma unroll
    for (int t = 0; t < kMaxRP; t++) {
        const int m = pb + t * 32 + lane;
        const bool in = t < p.rp && m < p.hc;
#pragma unroll
        for (int f = 0; f < NF; f++)
            v[f][t] = in ? __ldg(p.f[f] + rowoff + m) : make_float2(0.f, 0.f);
    }
}

// Registers -> the warp's staging buffer, with the two special modes fixed:
// (0,0,0) is skipped (zeroed) and the exact corner value replaces the
// transform's (N/2,N/2,N/2) mode.
template <int NF>
__device__ __forceinline__ void stage_piece(const BinParams &p, int64_t r, int pb, int lane,
                                            float2 (&v)[NF][kMaxRP], float2 *buf, int piece)
{
    if (r == 0 && pb == 0 && lane == 0) {
#pragma unroll
        for (int f = 0; f < NF; f++)
            v[f][0] = make_float2(0.f, 0.f);
    }
    if (r == p.corner_row) {
#pragma unroll
        for (int t = 0; t < kMaxRP; t++) {
            if (pb + t * 32 + lane == p.half) {
#pragma unroll
                for (int f = 0; f < NF; f++)
                    if (p.corner[f])
                        v[f][t] = make_float2((float)*p.corner[f], 0.f);
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < kMaxRP; t++) {
        if (t < p.rp) {
#pragma unroll
            for (int f = 0; f < NF; f++)
                buf[f * piece + t * 32 + lane] = v[f][t];
        }
    }
    __syncwarp();
}

// Work split: each warp takes a contiguous block of (i, j) rows; a row is
// walked in pieces of 32*RP modes, the next piece's loads in flight while the
// current one is binned.  Lane l bins the contiguous run [l*RP, (l+1)*RP) of a
// piece (RP odd: conflict-free strided shared reads) with a running FP32 sum
// per spectrum pair.  Along a run |k|^2 grows, so the bin only moves up: the
// next threshold is kept in a register and a completed bin inside a run is
// added to the warp's FP32 histogram with a shared atomic (rare: only where
// bins are narrower than a run).  At the end of a piece the lanes' open sums
// are combined by a segmented warp scan over their (non-decreasing) bins and
// each bin's last lane adds the total without atomics.  Every kPromoteRows
// rows the touched FP32 bins are promoted into the warp's FP64 histogram.
template <int NF, bool CROSS1>
__global__ void __launch_bounds__(256)
    k_bin(BinParams p, const uint32_t *__restrict__ thr_g, const float *__restrict__ iw_g,
          double *__restrict__ partial)
{
    constexpr int NP = PairSet<NF, CROSS1>::NP;
    extern __shared__ __align__(16) unsigned char smem[];
    const int nrb = p.nrbins;
    const int rp = p.rp, piece = 32 * rp;
    const BinLayout L = bin_layout(nrb, p.hc, NP, NF, rp);
    uint32_t *thr = (uint32_t *)smem;
    float2 *izc = (float2 *)(smem + L.izc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *wbase = smem + L.warps + L.per_warp * wid;
    double *whist = (double *)(wbase + L.whist);
    float *rhist = (float *)(wbase + L.rhist);
    float2 *buf = (float2 *)(wbase + L.buf);

    for (int i = threadIdx.x; i <= nrb; i += blockDim.x)
        thr[i] = thr_g[i];  // thr[nrb] = 0xffffffff: the bin never runs past nrb-1
    for (int i = threadIdx.x; i < p.hc; i += blockDim.x)
        izc[i] = make_float2(iw_g[i], (i == 0 || i == p.half) ? 1.f : 2.f);
    for (int i = lane; i < NP * nrb; i += 32) {
        whist[i] = 0.0;
        rhist[i] = 0.f;
    }
    __syncthreads();

    const int64_t nrows = (int64_t)p.dims * p.dims;
    const int64_t gw = (int64_t)blockIdx.x * p.warps + wid;
    const int64_t nw = (int64_t)gridDim.x * p.warps;
    const int64_t per = (nrows + nw - 1) / nw;
    const int64_t r_begin = min(nrows, gw * per), r_end = min(nrows, r_begin + per);
    int i = (int)(r_begin / p.dims), j = (int)(r_begin - (int64_t)i * p.dims);
    int bmin = nrb, bmax = -1;  // bins touched since the last FP64 promotion
    int rows_since = 0;
    float2 v[NF][kMaxRP];
    if (r_begin < r_end)
        load_piece<NF>(p, r_begin, 0, lane, v);
    for (int64_t r = r_begin; r < r_end; r++) {
        const int ki = kval_dev(i, p.dims), kj = kval_dev(j, p.dims);
        const uint32_t r2 = (uint32_t)(ki * ki + kj * kj);
        const float pxy = __ldg(iw_g + i) * __ldg(iw_g + j);
        for (int pb = 0; pb < p.hc; pb += piece) {
            stage_piece<NF>(p, r, pb, lane, v, buf, piece);
            // next piece (this row's, or the next row's first) in flight
            if (pb + piece < p.hc)
                load_piece<NF>(p, r, pb + piece, lane, v);
            else if (r + 1 < r_end)
                load_piece<NF>(p, r + 1, 0, lane, v);

            const int kz0 = pb + lane * rp;
            int cb = nrb;  // key of a lane without modes: sorts after every bin
            float acc[NP];
#pragma unroll
            for (int s = 0; s < NP; s++)
                acc[s] = 0.f;
            if (kz0 < p.hc) {
                uint32_t kk2 = r2 + (uint32_t)(kz0 * kz0);
                cb = bin_lookup(kk2, thr, nrb, p.bpu_half);
                bmin = min(bmin, cb);
                uint32_t nx = thr[cb + 1];
                const int lim = min(rp, p.hc - kz0);
                const float2 *bl = buf + lane * rp;
                for (int t = 0; t < lim; t++) {
                    const int kz = kz0 + t;
                    if (kk2 >= nx) {
#pragma unroll
                        for (int s = 0; s < NP; s++) {
                            atomicAdd(&rhist[s * nrb + cb], acc[s]);
                            acc[s] = 0.f;
                        }
                        do {
                            cb++;
                            nx = thr[cb + 1];
                        } while (kk2 >= nx);
                    }
                    const float2 ic = izc[kz];
                    const float pz = pxy * ic.x;
                    const float p2 = pz * pz;
                    const float w = ic.y * (p2 * p2);
                    float2 fv[NF];
#pragma unroll
                    for (int f = 0; f < NF; f++)
                        fv[f] = bl[f * piece + t];
                    add_pairs<NF, CROSS1>(fv, w, acc);
                    kk2 += (uint32_t)(2 * kz + 1);
                }
                bmax = max(bmax, cb);
            }
            // Segmented inclusive scan over lanes with equal open bin.
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int ku = __shfl_up_sync(0xffffffffu, cb, o);
#pragma unroll
                for (int s = 0; s < NP; s++) {
                    const float x = __shfl_up_sync(0xffffffffu, acc[s], o);
                    if (lane >= o && ku == cb)
                        acc[s] += x;
                }
            }
            const int kd = __shfl_down_sync(0xffffffffu, cb, 1);
            if (cb < nrb && (lane == 31 || kd != cb)) {
#pragma unroll
                for (int s = 0; s < NP; s++)
                    rhist[s * nrb + cb] += acc[s];
            }
            __syncwarp();
        }
        if (++j == p.dims) {
            j = 0;
            i++;
        }
        if (++rows_since == kPromoteRows || r + 1 == r_end) {
            rows_since = 0;
            const int lo = (int)__reduce_min_sync(0xffffffffu, (unsigned)bmin);
            const int hi = (int)__reduce_max_sync(0xffffffffu, (unsigned)(bmax + 1)) - 1;
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
            const double *wh = (const double *)(smem + L.warps + L.per_warp * w + L.whist);
            s += wh[k];
        }
        partial[(size_t)blockIdx.x * p.np * nrb + k] = s;
    }
}

// ---- binning of a kz-major spectrum (the N = 1024 transform) --------------
//
// The spectrum is stored as S[kz][x][y] (kz = 0..N/2, planes of N x N complex
// values; xfft.cu k_zfft_t1024 + a batched 2-D C2C).  Each (kz, x) row of N
// modes along y is binned as two half-rows along which |k|^2 grows: y = 0..N/2
// (ky = y) and y = N-1 down to N/2+1 (ky = y - N, |ky| = 1..N/2-1).  The rest
// is k_bin's: lane runs of RP modes with a running FP32 sum and the next
// threshold in a register, a segmented warp scan of the lanes' open sums,
// FP64 promotion every kPromoteRows half-rows, one FP64 partial histogram per
// CTA, k_bin_finalize.  Per mode: weight c = 1 on the kz = 0 and kz = N/2
// planes, 2 elsewhere; value c * p^4 |F|^2 with p = (iw_x iw_y) iw_z, the
// float product order of k_bin; (0,0,0) skipped; the exact corner value at
// (N/2, N/2, N/2).  One spectrum (its auto pair).
struct BinKzParams {
    const float2 *f;
    const double *corner;  // exact (N/2, N/2, N/2) value, or null
    int dims, half, hc;
    int nrbins;
    float bpu_half;
    int rp;     // modes per lane per piece (odd)
    int warps;  // warps per CTA
    uint4 *zero;          // region to clear (16-byte units), or null
    int64_t zero_units;
    int64_t zero_per_row; // units cleared per half-row
};

// Half-row r (physical row r/2 = kz * N + x, half r & 1): piece loads.
__device__ __forceinline__ void load_piece_kz(const BinKzParams &p, int64_t r, int pb, int lane,
                                              float2 (&v)[kMaxRP])
{
    const int h = (int)(r & 1);
    const int len = h ? p.half - 1 : p.hc;
    const float2 *row = p.f + (size_t)(r >> 1) * (size_t)p.dims;
#pragma unroll
    for (int t = 0; t < kMaxRP; t++) {
        const int m = pb + t * 32 + lane;
        const bool in = t < p.rp && m < len;
        const int y = h ? p.dims - 1 - m : m;
        v[t] = in ? __ldg(row + y) : make_float2(0.f, 0.f);
    }
}

__global__ void __launch_bounds__(256)
    k_bin_kz(BinKzParams p, const uint32_t *__restrict__ thr_g, const float *__restrict__ iw_g,
             double *__restrict__ partial)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int nrb = p.nrbins;
    const int rp = p.rp, piece = 32 * rp;
    const BinLayout L = bin_layout(nrb, p.hc, 1, 1, rp);
    uint32_t *thr = (uint32_t *)smem;
    float *iwy = (float *)(smem + L.izc);  // [dims]: 4 dims bytes fit the layout's 8 hc
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *wbase = smem + L.warps + L.per_warp * wid;
    double *whist = (double *)(wbase + L.whist);
    float *rhist = (float *)(wbase + L.rhist);
    float2 *buf = (float2 *)(wbase + L.buf);

    for (int i = threadIdx.x; i <= nrb; i += blockDim.x)
        thr[i] = thr_g[i];
    for (int i = threadIdx.x; i < p.dims; i += blockDim.x)
        iwy[i] = iw_g[i];
    for (int i = lane; i < nrb; i += 32) {
        whist[i] = 0.0;
        rhist[i] = 0.f;
    }
    __syncthreads();

    const int64_t nrows = (int64_t)2 * p.hc * p.dims;  // half-rows
    const int64_t gw = (int64_t)blockIdx.x * p.warps + wid;
    const int64_t nw = (int64_t)gridDim.x * p.warps;
    const int64_t per = (nrows + nw - 1) / nw;
    const int64_t r_begin = min(nrows, gw * per), r_end = min(nrows, r_begin + per);
    int bmin = nrb, bmax = -1;
    int rows_since = 0;
    float2 v[kMaxRP];
    if (r_begin < r_end)
        load_piece_kz(p, r_begin, 0, lane, v);
    for (int64_t r = r_begin; r < r_end; r++) {
        const int h = (int)(r & 1);
        const int64_t pr = r >> 1;
        const int kz = (int)(pr / p.dims), x = (int)(pr - (int64_t)kz * p.dims);
        const int kx = kval_dev(x, p.dims);
        const uint32_t r2 = (uint32_t)(kx * kx + kz * kz);
        const float cw = (kz == 0 || kz == p.half) ? 1.f : 2.f;
        const float iwx = iwy[x], iwz = iwy[kz];
        const int len = h ? p.half - 1 : p.hc;
        const bool origin = kz == 0 && x == 0 && h == 0;
        const bool corner = p.corner && kz == p.half && x == p.half && h == 0;
        if (p.zero) {  // this half-row's share of the clear (nothing waits on it)
            const int64_t a0 = r * p.zero_per_row;
            const int64_t e0 = min(a0 + p.zero_per_row, p.zero_units);
            for (int64_t u = a0 + lane; u < e0; u += 32)
                __stcs(p.zero + u, make_uint4(0u, 0u, 0u, 0u));
        }
        for (int pb = 0; pb < len; pb += piece) {
            if (origin && pb == 0 && lane == 0)
                v[0] = make_float2(0.f, 0.f);
            if (corner) {
#pragma unroll
                for (int t = 0; t < kMaxRP; t++)
                    if (pb + t * 32 + lane == p.half)
                        v[t] = make_float2((float)*p.corner, 0.f);
            }
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kMaxRP; t++)
                if (t < rp)
                    buf[t * 32 + lane] = v[t];
            __syncwarp();
            if (pb + piece < len)
                load_piece_kz(p, r, pb + piece, lane, v);
            else if (r + 1 < r_end)
                load_piece_kz(p, r + 1, 0, lane, v);

            const int m0 = pb + lane * rp;
            int cb = nrb;
            float acc = 0.f;
            if (m0 < len) {
                int ky = m0 + h;  // |ky| of the run's first mode
                uint32_t kk2 = r2 + (uint32_t)(ky * ky);
                cb = bin_lookup(kk2, thr, nrb, p.bpu_half);
                bmin = min(bmin, cb);
                uint32_t nx = thr[cb + 1];
                const int lim = min(rp, len - m0);
                const float2 *bl = buf + lane * rp;
                for (int t = 0; t < lim; t++) {
                    if (kk2 >= nx) {
                        atomicAdd(&rhist[cb], acc);
                        acc = 0.f;
                        do {
                            cb++;
                            nx = thr[cb + 1];
                        } while (kk2 >= nx);
                    }
                    const int m = m0 + t;
                    const int y = h ? p.dims - 1 - m : m;
                    const float pz = (iwx * iwy[y]) * iwz;
                    const float p2 = pz * pz;
                    const float w = cw * (p2 * p2);
                    const float2 fv = bl[t];
                    acc = fmaf(w, fmaf(fv.x, fv.x, fv.y * fv.y), acc);
                    kk2 += (uint32_t)(2 * ky + 1);
                    ky++;
                }
                bmax = max(bmax, cb);
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int ku = __shfl_up_sync(0xffffffffu, cb, o);
                const float xo = __shfl_up_sync(0xffffffffu, acc, o);
                if (lane >= o && ku == cb)
                    acc += xo;
            }
            const int kd = __shfl_down_sync(0xffffffffu, cb, 1);
            if (cb < nrb && (lane == 31 || kd != cb))
                rhist[cb] += acc;
            __syncwarp();
        }
        if (++rows_since == kPromoteRows || r + 1 == r_end) {
            rows_since = 0;
            const int lo = (int)__reduce_min_sync(0xffffffffu, (unsigned)bmin);
            const int hi = (int)__reduce_max_sync(0xffffffffu, (unsigned)(bmax + 1)) - 1;
            for (int b = lo + lane; b <= hi; b += 32) {
                whist[b] += (double)rhist[b];
                rhist[b] = 0.f;
            }
            __syncwarp();
            bmin = nrb;
            bmax = -1;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nrb; k += blockDim.x) {
        double sum = 0.0;
        for (int w = 0; w < p.warps; w++) {
            const double *wh = (const double *)(smem + L.warps + L.per_warp * w + L.whist);
            sum += wh[k];
        }
        partial[(size_t)blockIdx.x * nrb + k] = sum;
    }
}

struct NormParams {
    double ma[kMaxBinPairs], mb[kMaxBinPairs];
    int src[kMaxBinPairs];  // the partials' pair slot of each reported pair
    int npc;                // pair slots per CTA partial
};

// One block per (pair, bin): strided sums over the CTA partials, then a
// fixed-order tree, so the result does not depend on scheduling.
constexpr int kFinalizeThreads = 256;

__global__ void __launch_bounds__(kFinalizeThreads)
    k_bin_finalize(const double *__restrict__ partial, int ctas, int nrbins,
                   const double *__restrict__ count, NormParams mn, double *__restrict__ power,
                   const DeviceStatus *__restrict__ st_in, DeviceStatus *__restrict__ st_out)
{
    if (st_out && blockIdx.x == 0 && threadIdx.x == 0)
        *st_out = *st_in;  // the pass's status words, beside the results
    __shared__ double sh[kFinalizeThreads];
    const int k = blockIdx.x;
    const int s = k / nrbins, b = k - s * nrbins;
    const size_t src = (size_t)mn.src[s] * nrbins + b;
    double part = 0.0;
    for (int c = threadIdx.x; c < ctas; c += blockDim.x)
        part += partial[(size_t)c * mn.npc * nrbins + src];
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

int bin_rp(int hc)
{
    return hc <= 32 ? 1 : hc <= 96 ? 3 : hc <= 160 ? 5 : 9;
}

size_t bin_smem(int nrbins, int hc, int np, int nf, int warps)
{
    const BinLayout L = bin_layout(nrbins, hc, np, nf, bin_rp(hc));
    return L.warps + L.per_warp * warps;
}

// Instantiated shapes: one field (its auto pair); two fields and one pair
// (the cross pair alone); else every pair of 2, 3 or 4 fields.  A request's
// pairs are found among the shape's by pair_slot.
struct Shape {
    int nf, np;
    bool cross1;
};

Shape pick_shape(int nf, int np)
{
    if (nf == 1)
        return {1, 1, false};
    if (nf == 2 && np == 1)
        return {2, 1, true};
    if (nf >= 2 && nf <= kMaxBinFields)
        return {nf, nf * (nf + 1) / 2, false};
    return {0, 0, false};
}

}  // namespace

int bin_pair_slots(int nfields, int npairs)
{
    return pick_shape(nfields, npairs).np;
}

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
                        int warps, size_t smem, cudaStream_t stream, int64_t *launches,
                        const DeviceStatus *st_in, DeviceStatus *st_out)
{
    const Shape s = pick_shape(l.nfields, l.npairs);
    BinParams p;
    for (int f = 0; f < kMaxBinFields; f++) {
        p.f[f] = l.fields[f < l.nfields ? f : 0];
        p.corner[f] = l.corner[f < l.nfields ? f : 0];
    }
    p.corner_row = (g.dims % 2 == 0) ? (int64_t)g.half * g.dims + g.half : -1;
    p.np = s.np;
    p.dims = g.dims;
    p.hc = g.hc;
    p.half = g.half;
    p.nrbins = t.nrbins;
    p.bpu_half = (float)(0.5 * t.binsperunit);
    p.rp = bin_rp(g.hc);
    p.warps = warps;
    cudaError_t err;
#define GENPK_BIN_LAUNCH(NF, CROSS1)                                                          \
    do {                                                                                      \
        auto kern = k_bin<NF, CROSS1>;                                                        \
        if ((err = ensure_dynamic_smem(kern, smem)) != cudaSuccess)                           \
            return err;                                                                       \
        kern<<<ctas, 32 * warps, smem, stream>>>(p, d.thr, d.iw, partial);                    \
    } while (0)
    if (s.nf == 1)
        GENPK_BIN_LAUNCH(1, false);
    else if (s.nf == 2 && s.cross1)
        GENPK_BIN_LAUNCH(2, true);
    else if (s.nf == 2)
        GENPK_BIN_LAUNCH(2, false);
    else if (s.nf == 3)
        GENPK_BIN_LAUNCH(3, false);
    else
        GENPK_BIN_LAUNCH(4, false);
#undef GENPK_BIN_LAUNCH
    (*launches)++;
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    NormParams mn;
    mn.npc = s.np;
    for (int q = 0; q < kMaxBinPairs; q++) {
        mn.ma[q] = q < l.npairs ? l.pairs[q].mass_a : 1.0;
        mn.mb[q] = q < l.npairs ? l.pairs[q].mass_b : 1.0;
        const int a = q < l.npairs ? std::min(l.pairs[q].a, l.pairs[q].b) : 0;
        const int b = q < l.npairs ? std::max(l.pairs[q].a, l.pairs[q].b) : 0;
        mn.src[q] = s.cross1 ? 0 : pair_slot(s.nf, a, b);
    }
    const int k = l.npairs * t.nrbins;
    k_bin_finalize<<<k, kFinalizeThreads, 0, stream>>>(partial, ctas, t.nrbins, d.count, mn,
                                                        out_power, st_in, st_out);
    (*launches)++;
    return cudaGetLastError();
}

int bin_kz_ctas(const GridGeom &g, int nrbins, int num_sms, int *warps, size_t *smem)
{
    int w = 8;
    while (w > 1 && bin_smem(nrbins, g.hc, 1, 1, w) > 200 * 1024)
        w /= 2;
    const size_t sm = bin_smem(nrbins, g.hc, 1, 1, w);
    if (sm > 220 * 1024 || (size_t)4 * g.dims > align16(sizeof(float2) * g.hc))
        return 0;
    *warps = w;
    *smem = sm;
    const int per_sm = std::max(1, std::min(2048 / (32 * w), (int)((220 * 1024) / sm)));
    const int64_t rows = (int64_t)2 * g.hc * g.dims;
    const int64_t want = (rows + w - 1) / w;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms * per_sm, want));
}

cudaError_t bin_spectrum_kz(const GridGeom &g, const BinTables &t, const BinDevice &d,
                            const float2 *spec, const double *corner, double *partial, int ctas,
                            int warps, size_t smem, void *zero, int64_t zero_bytes,
                            cudaStream_t stream, int64_t *launches)
{
    BinKzParams p;
    p.f = spec;
    p.corner = (g.dims % 2 == 0) ? corner : nullptr;
    p.dims = g.dims;
    p.half = g.half;
    p.hc = g.hc;
    p.nrbins = t.nrbins;
    p.bpu_half = (float)(0.5 * t.binsperunit);
    p.rp = bin_rp(g.hc);
    p.warps = warps;
    p.zero = reinterpret_cast<uint4 *>(zero);
    p.zero_units = zero ? zero_bytes / 16 : 0;
    const int64_t half_rows = (int64_t)2 * g.hc * g.dims;
    p.zero_per_row = (p.zero_units + half_rows - 1) / half_rows;
    cudaError_t err;
    if ((err = ensure_dynamic_smem(k_bin_kz, smem)) != cudaSuccess)
        return err;
    k_bin_kz<<<ctas, 32 * warps, smem, stream>>>(p, d.thr, d.iw, partial);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t finalize_power(const double *partial, int ctas, int nrbins, const double *count,
                           double ma, double mb, double *out, cudaStream_t stream,
                           int64_t *launches, const DeviceStatus *st_in, DeviceStatus *st_out)
{
    NormParams mn;
    mn.npc = 1;
    for (int q = 0; q < kMaxBinPairs; q++) {
        mn.ma[q] = q == 0 ? ma : 1.0;
        mn.mb[q] = q == 0 ? mb : 1.0;
        mn.src[q] = 0;
    }
    k_bin_finalize<<<nrbins, kFinalizeThreads, 0, stream>>>(partial, ctas, nrbins, count, mn,
                                                            out, st_in, st_out);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t finalize_powers(const double *partial, int ctas, int nrbins, int nfields,
                            const double *count, const double *mass, double *out,
                            cudaStream_t stream, int64_t *launches, const DeviceStatus *st_in,
                            DeviceStatus *st_out)
{
    for (int f0 = 0; f0 < nfields; f0 += kMaxBinPairs) {
        const int k = std::min(kMaxBinPairs, nfields - f0);
        NormParams mn;
        mn.npc = nfields;
        for (int q = 0; q < kMaxBinPairs; q++) {
            mn.ma[q] = mn.mb[q] = q < k ? mass[f0 + q] : 1.0;
            mn.src[q] = q < k ? f0 + q : 0;
        }
        const bool last = f0 + k >= nfields;
        k_bin_finalize<<<k * nrbins, kFinalizeThreads, 0, stream>>>(
            partial, ctas, nrbins, count, mn, out + (size_t)f0 * nrbins, st_in,
            last ? st_out : nullptr);
        (*launches)++;
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess)
            return err;
    }
    return cudaSuccess;
}

}  // namespace genpk
