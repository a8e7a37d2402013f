// deposit_window.cu -- CIC deposit for spatially coherent particle order.
//
// N-body snapshots usually store particles in a spatially coherent order:
// initial-condition lattice order (the Zel'dovich sets used here), or the
// Peano-Hilbert order of a simulation's domain decomposition.  Then every
// contiguous run of a few thousand particles occupies a small region of the
// grid, and the tile sort in deposit.cu is unnecessary work.  This engine:
//
//   k_window_deposit  persistent: one CTA per SM walks chunks of `chunk`
//     consecutive particles (chunk b, b + gridDim, ...); the chunk length
//     (4096 down to 512) is the largest whose sampled windows fit, a smaller
//     chunk leaving more shared memory to the window.  Chunks arrive in
//     shared memory by bulk asynchronous copy (cp.async.bulk + mbarrier),
//     double-buffered so the next chunk streams in while this one is worked.
//     pass A  finds the periodic bounding box of the chunk's cells (cells from
//             a plain FP32 product, one cell off for a few positions next to a
//             cell face: pass B sends those, if they fall outside the box,
//             down the global path); an axis the chunk spans completely is
//             taken whole, with one extra layer for the wrapped CIC corner.
//             Invalid particles are counted and marked (x := NaN).
//     pass B  splits every position exactly (split_q28) and adds the eight
//             CIC weights (at most 2^28 units each) to the shared window with
//             native shared integer atomics; a signed overflow of a window
//             cell adds +-2^32 to its grid cell.  Pass B also sums the chunk's
//             share of the exact corner mode.
//     flush   every non-zero window cell is added to the 64-bit pass
//             accumulator (global RED, no return) and cleared, so the window
//             is zero again for the next chunk.
//
//   k_stream_deposit  the stream mode: the same chunk pipeline without the
//     window, for lattice order at about one particle per cell (where windows
//     merge few adds); each particle's weights go to the accumulator as L2
//     reductions, merged between neighbouring lanes of one z cell column.
//     Chosen by the merge rate k_stream_probe measures.
//
// Sums are exact: the window cells (32-bit, overflows moved on as 2^32 units)
// and the pass accumulator (64-bit) are integers of 2^-s mass units (the
// sorted engine's weights, common.cuh pair_w / z_mass / corner_w);
// k_window_convert subtracts the fixed-point pass mean and rounds each cell
// once to FP32 (or the forward transform's z pass does the same as it reads
// the accumulator, xfft.cu k_zfft).  The grid is therefore bit-identical to
// the sorted engine's, in either mode, and independent of summation order.
// The accumulator is zeroed before each pass: by a memset here, or already by
// the binning x pass of the spectrum that used its previous contents.
#include "bulk.cuh"
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <cstdlib>
#include <type_traits>

namespace genpk {
namespace {

constexpr int kWinThreads = 1024;
constexpr int kWinSmemBytes = 225 * 1024;     // dynamic shared memory per CTA
constexpr float kPosLimit = 1.0e9f;           // |pos * units| above this: invalid

struct WinParams {
    const float *pos;
    const float *masses;
    int64_t n;
    int64_t nchunks;
    int chunk;
    int cap;      // window capacity in cells
    int win_off;  // byte offset of the window in dynamic shared memory
    int dims;
    float fdims, inv_dims;
    float uh, ul;
    float umass;
    int64_t plane;
    int row;
    int corner;  // accumulate the exact (N/2,N/2,N/2) mode (even grids)
    int bulk;    // positions (and masses) 16-byte aligned: full chunks by bulk copy
    // Testing aid (genpk_inject_copy_timeout): the bulk copy of chunk
    // skip_chunk is not issued and the wait for it gives up after skip_wait
    // clocks; -1 for none.
    int64_t skip_chunk;
    long long skip_wait;
    // A uniform mass's pass constants, computed on the host (host_prep = 1) as
    // k_window_prep computes them; thread 0 of CTA 0 stores them in the status
    // words and adds the pass to the grid's running sums.  Else (host_prep = 0)
    // k_window_prep ran before the pass.
    int host_prep;
    int fx_shift;
    double pass_mass;
    long long mean_fixed;
    double *field_mass, *field_sub;
};

// The pass constants of k_window_prep, on the host for a uniform mass (the
// same IEEE operations in the same order: the same bits).
struct PassConsts {
    double mass;
    int fx_shift;
    long long mean_fixed;
};

__host__ __device__ inline PassConsts pass_consts(double m, float mref, double inv_cells)
{
    int s = 0;
    if (mref > 0.f && isfinite(mref))
        s = 27 - ilogbf(mref);
    s = max(-100, min(100, s));
    const double mf = m * inv_cells * ldexp(1.0, s);
    long long mean_fixed;
    const double amf = fabs(mf);
    if (amf >= 16777216.0) {
        const double q = ldexp(1.0, ilogb(amf) - 23);
        mean_fixed = (long long)(rint(mf / q) * q);
    } else {
        mean_fixed = llrint(mf);
    }
    return {m, s, mean_fixed};
}

// Thread 0 of CTA 0: the host-computed constants into the status words and
// the grid's running sums (a uniform-mass pass without k_window_prep).
__device__ __forceinline__ void store_host_prep(const WinParams &p, DeviceStatus *st)
{
    if (p.host_prep && blockIdx.x == 0 && threadIdx.x == 0) {
        st->pass_mass = p.pass_mass;
        st->fx_shift = p.fx_shift;
        st->mean_fixed = p.mean_fixed;
        *p.field_mass += p.pass_mass;
        *p.field_sub += ldexp((double)p.mean_fixed, -p.fx_shift);
    }
}

// ---- helpers ---------------------------------------------------------------

__device__ __forceinline__ int wrap_once(int v, int n)
{
    return v < 0 ? v + n : (v >= n ? v - n : v);
}

// Integer-valued float cell in [0, dims) near position v along one axis; 0
// for an invalid position.  Only needs to be close to the chunk's particles.
__device__ __forceinline__ float ref_cell(const WinParams &p, float v)
{
    float r = floorf(v * p.uh);
    r = fmaf(-p.fdims, floorf(r * p.inv_dims), r);
    return (r >= 0.f && r < p.fdims) ? r : 0.f;
}

struct WinBox {
    int org[3];
    int ext[3];  // window extent per axis (cells)
    bool use;    // the box fits the window
};

// Block-wide periodic bounding box from the per-thread float offset ranges
// [fmn, fmx] (offsets from ref; empty when fmn > fmx).  Two barriers.
__device__ __forceinline__ WinBox window_box(const float fmn[3], const float fmx[3],
                                             const float ref[3], const WinParams &p,
                                             int (*sh_mm)[32], int *sh_box)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned bias = 1u << 30;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int lo = fmn[a] <= fmx[a] ? (int)floorf(fmaxf(fmn[a], -1.0e9f)) : (1 << 29);
        const int hi = fmn[a] <= fmx[a] ? (int)floorf(fminf(fmx[a], 1.0e9f)) : -(1 << 29);
        const unsigned rlo = __reduce_min_sync(0xffffffffu, (unsigned)(lo + (int)bias));
        const unsigned rhi = __reduce_max_sync(0xffffffffu, (unsigned)(hi + (int)bias));
        if (lane == 0) {
            sh_mm[a][wid] = (int)(rlo - bias);
            sh_mm[3 + a][wid] = (int)(rhi - bias);
        }
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        long long vol = 1;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int lo = lane < nw ? sh_mm[a][lane] : (1 << 29);
            const int hi = lane < nw ? sh_mm[3 + a][lane] : -(1 << 29);
            const int mlo = (int)(__reduce_min_sync(0xffffffffu, (unsigned)(lo + (int)bias)) - bias);
            const int mhi = (int)(__reduce_max_sync(0xffffffffu, (unsigned)(hi + (int)bias)) - bias);
            int org, ext;
            if (mhi < mlo) {  // no valid particle
                org = 0;
                ext = 1;
            } else if (mhi - mlo + 2 >= p.dims) {  // the whole axis (+1 wrapped layer)
                org = 0;
                ext = p.dims + 1;
            } else {  // +1 for the CIC corner
                org = wrap_once((int)ref[a] + mlo, p.dims);
                ext = mhi - mlo + 2;
            }
            if (lane == 0) {
                sh_box[a] = org;
                sh_box[3 + a] = ext;
            }
            vol *= ext;
        }
        if (lane == 0)
            sh_box[6] = vol <= p.cap ? 1 : 0;
    }
    __syncthreads();
    WinBox b;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        b.org[a] = sh_box[a];
        b.ext[a] = sh_box[3 + a];
    }
    b.use = sh_box[6] != 0;
    return b;
}

__device__ __forceinline__ int64_t chunk_first(const WinParams &p, int64_t c)
{
    return c * (int64_t)p.chunk;
}

__device__ __forceinline__ bool chunk_by_bulk(const WinParams &p, int64_t c)
{
    return p.bulk && (c + 1) * (int64_t)p.chunk <= p.n;
}

// One thread: bulk copies of chunk c into (P, M), completing on `bar`.
template <bool VARMASS>
__device__ __forceinline__ void issue_chunk(const WinParams &p, int64_t c, float *P, float *M,
                                            unsigned long long *bar)
{
    if (c == p.skip_chunk)  // testing aid: no copy, so the wait for it runs out
        return;
    const unsigned pb = (unsigned)p.chunk * 12u, mb = VARMASS ? (unsigned)p.chunk * 4u : 0u;
    fence_proxy_async();
    mbar_expect_tx(bar, pb + mb);
    bulk_load(P, p.pos + 3 * chunk_first(p, c), pb, bar);
    if (VARMASS)
        bulk_load(M, p.masses + chunk_first(p, c), mb, bar);
}

// All threads: n floats src -> dst (dst 16-byte aligned), 16 bytes at a time
// where src allows.
__device__ __forceinline__ void copy_floats(float *dst, const float *src, int n)
{
    int done = 0;
    if (((uintptr_t)src & 15u) == 0u) {
        const int n4 = n >> 2;
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
        for (int i = threadIdx.x; i < n4; i += blockDim.x)
            d4[i] = s4[i];
        done = n4 << 2;
    }
    for (int i = done + threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
}

// All threads: plain copy of chunk c (tail chunk, unaligned input, or pinned
// host memory read in place).
template <bool VARMASS>
__device__ __forceinline__ void copy_chunk(const WinParams &p, int64_t c, int cnt, float *P,
                                           float *M)
{
    copy_floats(P, p.pos + 3 * chunk_first(p, c), 3 * cnt);
    if (VARMASS)
        copy_floats(M, p.masses + chunk_first(p, c), cnt);
}

// Chunk arrival, every thread.  A bulk-copied chunk (bulk) is waited for on
// bar's phase `parity`, with a bounded wait; any other chunk is loaded with
// plain loads.  Ends with a barrier: the chunk is in place and every thread is
// done with the other buffer.  If the wait ran out on any thread, the whole
// CTA (the decision is made at the barrier, so it is uniform) waits once more,
// bounded, for a copy that may still be in flight, counts one timeout, loads
// the chunk with plain loads and sets `broken`: this CTA issues no further bulk
// copies (the barrier's phase may never complete), so the pass still deposits
// every particle and only its status reports the wait.
template <bool VARMASS>
__device__ __forceinline__ void arrive_chunk(const WinParams &p, int64_t c, int cnt, bool bulk,
                                             float *P, float *M, unsigned long long *bar,
                                             unsigned parity, bool &broken, unsigned &timeouts)
{
    const long long limit = c == p.skip_chunk ? p.skip_wait : kWaitClocks;
    bool late = false;
    if (bulk)
        late = !mbar_wait(bar, parity, limit);
    else
        copy_chunk<VARMASS>(p, c, cnt, P, M);
    if (__syncthreads_or(late)) {
        mbar_wait(bar, parity, limit);
        __syncthreads();
        copy_chunk<VARMASS>(p, c, cnt, P, M);
        __syncthreads();
        broken = true;
        if (threadIdx.x == 0)
            timeouts++;
    }
}

// The pass accumulates exact 64-bit integers acc[gi] for every padded grid
// index gi; adds return nothing (RED), so they never wait.
typedef unsigned long long acc_t;

__device__ __forceinline__ void acc_add_global(acc_t *acc, size_t gi, long long v)
{
    atomicAdd(acc + gi, (acc_t)v);
}

__device__ __forceinline__ size_t corner_index(const WinParams &p, const int c[3], int k)
{
    const int x = (k & 1) ? (c[0] + 1 == p.dims ? 0 : c[0] + 1) : c[0];
    const int y = (k & 2) ? (c[1] + 1 == p.dims ? 0 : c[1] + 1) : c[1];
    const int z = (k & 4) ? (c[2] + 1 == p.dims ? 0 : c[2] + 1) : c[2];
    return cell_index(p.plane, p.row, x, y, z);
}

// Global-path adds of one particle's eight corners (cells c, signed weights
// w[k] for corner k = dx | dy << 1 | dz << 2).
__device__ __noinline__ void global_corners(const WinParams &p, acc_t *acc, const int c[3],
                                            const int w[8])
{
#pragma unroll
    for (int k = 0; k < 8; k++)
        if (w[k] != 0)
            acc_add_global(acc, corner_index(p, c, k), w[k]);
}

// Window cells of the corners in `mask` overflowed by `sign`: move +-2^32
// into their grid cells.
__device__ __noinline__ void carry_corners(const WinParams &p, acc_t *acc, const int c[3],
                                           unsigned mask, int sign)
{
#pragma unroll
    for (int k = 0; k < 8; k++)
        if ((mask >> k) & 1u)
            acc_add_global(acc, corner_index(p, c, k), (long long)sign << 32);
}

// Block epilogue of both deposit kernels: the warps' shares of the exact
// corner mode (fixed point, 2^-(s+4) units) and the invalid-particle and
// wait-timeout counts.
template <bool VARMASS, bool CORNER>
__device__ __forceinline__ void report_block(const WinParams &p, DeviceStatus *st, f2sum alt,
                                             unsigned bad, unsigned timeouts, float mscale)
{
    const int lane = threadIdx.x & 31;
    if (CORNER) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const f2sum other = {__shfl_xor_sync(0xffffffffu, alt.hi, o),
                                 __shfl_xor_sync(0xffffffffu, alt.lo, o)};
            alt = f2_add2(alt, other);
        }
        if (lane == 0) {
            if (!VARMASS) {  // the uniform mass was factored out of the sum
                const float mm = p.umass * mscale;
                const float h = __fmul_rn(alt.hi, mm);
                alt = f2sum{h, fmaf(alt.hi, mm, -h) + alt.lo * mm};
            }
            const long long v = __float2ll_rn(alt.hi) + __float2ll_rn(alt.lo);
            if (v != 0)
                atomicAdd((unsigned long long *)&st->alt_sum, (unsigned long long)v);
        }
    }
    bad = __reduce_add_sync(0xffffffffu, bad);
    timeouts = __reduce_add_sync(0xffffffffu, timeouts);
    if (lane == 0 && bad)
        atomicAdd(&st->bad_particles, (unsigned long long)bad);
    if (lane == 0 && timeouts)
        atomicAdd(&st->timeouts, (unsigned long long)timeouts);
}

template <bool VARMASS, bool CORNER>
__global__ void __launch_bounds__(kWinThreads, 1)
    k_window_deposit(WinParams p, DeviceStatus *st, acc_t *__restrict__ acc)
{
    extern __shared__ __align__(128) unsigned char win_smem[];
    float *pbuf = reinterpret_cast<float *>(win_smem);              // [2][chunk * 3]
    float *mbuf = pbuf + 6 * p.chunk;                               // [2][chunk] (VARMASS)
    int *win = reinterpret_cast<int *>(win_smem + p.win_off);       // [cap]
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ int sh_mm[6][32];
    __shared__ int sh_box[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;

    for (int i = threadIdx.x; i < p.cap; i += blockDim.x)
        win[i] = 0;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();

    // Weights in 2^-s mass units, s = 154 - emax (common.cuh pair_w / z_mass /
    // corner_w, as the sorted engine computes them).
    store_host_prep(p, st);
    const int fxs = p.host_prep ? p.fx_shift : st->fx_shift;
    const int emax = 154 - fxs;
    const unsigned ubits = __float_as_uint(p.umass);
    const unsigned umant = (ubits & 0x7fffffu) | 0x800000u;
    const int uef = (int)((ubits >> 23) & 0xffu);
    const bool uneg = (ubits >> 31) != 0u;
    const float mscale = ldexpf(1.f, fxs + 4);

    f2sum alt = {0.f, 0.f};
    unsigned bad = 0, timeouts = 0;
    bool broken = false;  // a wait ran out: plain loads from then on
    const int64_t c0 = blockIdx.x;
    if (threadIdx.x == 0 && c0 < p.nchunks && chunk_by_bulk(p, c0))
        issue_chunk<VARMASS>(p, c0, pbuf, mbuf, &bar[0]);

    int k = 0;
    for (int64_t c = c0; c < p.nchunks; c += gridDim.x, k++) {
        const int buf = k & 1;
        float *P = pbuf + buf * 3 * p.chunk;
        float *M = mbuf + buf * p.chunk;
        const int cnt = (int)min((int64_t)p.chunk, p.n - chunk_first(p, c));
        arrive_chunk<VARMASS>(p, c, cnt, !broken && chunk_by_bulk(p, c), P, M, &bar[buf],
                              (unsigned)(k >> 1) & 1u, broken, timeouts);

        // Pass A: float offsets of the approximate cells from the chunk's
        // first particle, periodic-wrapped into [-N/2, N/2].
        const float ref[3] = {ref_cell(p, P[0]), ref_cell(p, P[1]), ref_cell(p, P[2])};
        float fmn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, fmx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
            float f[3];
            bool ok = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                f[a] = fmaf(P[3 * j + a], p.uh, -ref[a]);
                ok = ok && fabsf(f[a]) <= kPosLimit;
            }
            if (VARMASS)
                ok = ok && fabsf(M[j]) <= 3.4028235e38f;
            if (!ok) {
                P[3 * j] = __int_as_float(0x7fffffff);
                fence_proxy_async();  // before a later bulk copy into this buffer
                bad++;
                continue;
            }
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float w = fmaf(-p.fdims, rintf(f[a] * p.inv_dims), f[a]);
                fmn[a] = fminf(fmn[a], w);
                fmx[a] = fmaxf(fmx[a], w);
            }
        }
        // Prefetch the chunk after this one into the other buffer (its last
        // reader, pass B of the previous chunk, finished before the previous
        // flush's barrier).
        if (threadIdx.x == 0 && !broken && c + gridDim.x < p.nchunks &&
            chunk_by_bulk(p, c + gridDim.x))
            issue_chunk<VARMASS>(p, c + gridDim.x, pbuf + (buf ^ 1) * 3 * p.chunk,
                                 mbuf + (buf ^ 1) * p.chunk, &bar[buf ^ 1]);
        const WinBox box = window_box(fmn, fmx, ref, p, sh_mm, sh_box);
        const int e0 = box.ext[0] - 1, e1 = box.ext[1] - 1, e2 = box.ext[2] - 1;
        const int DY = box.ext[2], DX = box.ext[1] * box.ext[2];

        // Pass B: exact split, fixed-point weights, corner-mode share.
        for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
            const float x = P[3 * j], y = P[3 * j + 1], z = P[3 * j + 2];
            if (isnan(x))
                continue;
            float m = p.umass;
            unsigned mant = umant;
            int ef = uef;
            bool neg = uneg;
            if (VARMASS) {
                m = M[j];
                const unsigned mb = __float_as_uint(m);
                ef = (int)((mb >> 23) & 0xffu);
                mant = (mb & 0x7fffffu) | 0x800000u;
                neg = (mb >> 31) != 0u;
            }
            if (ef == 0)  // zero or subnormal mass deposits nothing
                continue;
            const int dsh = max(emax - ef, 0);
            // The stream kernel's fast split where 1 <= |x N/L| < 2^22 cells on
            // every axis (the same cells and fractions as split_q28).
            const float xh = __fmul_rn(x, p.uh), yh = __fmul_rn(y, p.uh), zh = __fmul_rn(z, p.uh);
            AxisQ ax, ay, az;
            if (fabsf(xh) >= 1.f && fabsf(xh) < kFastSplitMax && fabsf(yh) >= 1.f &&
                fabsf(yh) < kFastSplitMax && fabsf(zh) >= 1.f && fabsf(zh) < kFastSplitMax) {
                ax = split_q28_unwrapped(x, xh, p.uh, p.ul);
                ay = split_q28_unwrapped(y, yh, p.uh, p.ul);
                az = split_q28_unwrapped(z, zh, p.uh, p.ul);
                if (max((unsigned)ax.cell, max((unsigned)ay.cell, (unsigned)az.cell)) >=
                    (unsigned)p.dims) {
                    ax.cell = wrap_cell(ax.cell, p.dims);
                    ay.cell = wrap_cell(ay.cell, p.dims);
                    az.cell = wrap_cell(az.cell, p.dims);
                }
            } else {
                ax = split_q28(x, p.uh, p.ul, p.dims);
                ay = split_q28(y, p.uh, p.ul, p.dims);
                az = split_q28(z, p.uh, p.ul, p.dims);
            }
            if (CORNER) {
                f2sum v = corner_factor_q(ax, ay, az);
                if (VARMASS) {
                    const float mm = m * mscale;
                    const float h = __fmul_rn(v.hi, mm);
                    v = f2sum{h, fmaf(v.hi, mm, -h) + v.lo * mm};
                }
                f2_accumulate(alt, f2_signed(v, ax.cell ^ ay.cell ^ az.cell));
            }
            // Weights (common.cuh): factors 2^28 - q (lower cell) and q (upper).
            const uint32_t rx = kFracOne - ax.q, ry = kFracOne - ay.q, rz = kFracOne - az.q;
            const uint32_t p00 = pair_w(rx, ry), p10 = pair_w(ax.q, ry), p01 = pair_w(rx, ay.q),
                           p11 = pair_w(ax.q, ay.q);
            const uint32_t z0 = z_mass(rz, mant, VARMASS ? dsh : 0);
            const uint32_t z1 = z_mass(az.q, mant, VARMASS ? dsh : 0);
            const uint32_t w[8] = {corner_w(p00, z0), corner_w(p10, z0), corner_w(p01, z0),
                                   corner_w(p11, z0), corner_w(p00, z1), corner_w(p10, z1),
                                   corner_w(p01, z1), corner_w(p11, z1)};
            const int cell[3] = {ax.cell, ay.cell, az.cell};
            int o0 = ax.cell - box.org[0], o1 = ay.cell - box.org[1], o2 = az.cell - box.org[2];
            o0 += o0 < 0 ? p.dims : 0;
            o1 += o1 < 0 ? p.dims : 0;
            o2 += o2 < 0 ? p.dims : 0;
            if (box.use && o0 < e0 && o1 < e1 && o2 < e2) {
                int *wp = win + (o0 * box.ext[1] + o1) * DY + o2;
                const int off[8] = {0, DX, DY, DX + DY, 1, DX + 1, DY + 1, DX + DY + 1};
                int old[8];
                unsigned any = 0u;
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    old[q] = atomicAdd(wp + off[q], neg ? -(int)w[q] : (int)w[q]);
                    any |= (unsigned)old[q];
                }
                // An add of |w| <= 2^28 can only overflow a cell that held at
                // least 2^31 - 2^28 or a negative value: test exactly only then.
                if (any >= 0x70000000u) {
                    unsigned ovf = 0u;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const int sw = neg ? -(int)w[q] : (int)w[q];
                        const int nw = (int)((unsigned)old[q] + (unsigned)sw);
                        ovf |= (unsigned)(neg ? nw > old[q] : nw < old[q]) << q;
                    }
                    if (ovf)
                        carry_corners(p, acc, cell, ovf, neg ? -1 : 1);
                }
            } else {
                int wi[8];
#pragma unroll
                for (int q = 0; q < 8; q++)
                    wi[q] = neg ? -(int)w[q] : (int)w[q];
                global_corners(p, acc, cell, wi);
            }
        }
        __syncthreads();

        // Flush and clear: one warp per window row, lanes along z (each
        // reduction instruction then covers consecutive cells); every non-zero
        // cell is added exactly to the pass accumulator.
        if (box.use) {
            const int nrows = box.ext[0] * box.ext[1];
            for (int r = wid; r < nrows; r += nwarps) {
                const int wx = r / box.ext[1];
                const int wy = r - wx * box.ext[1];
                const int gx = wrap_once(box.org[0] + wx, p.dims);
                const int gy = wrap_once(box.org[1] + wy, p.dims);
                acc_t *arow = acc + (size_t)gx * (size_t)p.plane + (size_t)gy * (size_t)p.row;
                int *wrow = win + (size_t)r * DY;
                for (int z = lane; z < box.ext[2]; z += 32) {
                    const int v = wrow[z];
                    if (v != 0) {
                        wrow[z] = 0;
                        int gz = box.org[2] + z;
                        gz -= gz >= p.dims ? p.dims : 0;
                        atomicAdd(arow + gz, (acc_t)(long long)v);
                    }
                }
            }
        }
        // The next chunk's window writes come after the two barriers of its
        // window_box, so the flush needs no barrier of its own.
    }

    report_block<VARMASS, CORNER>(p, st, alt, bad, timeouts, mscale);
}

// Stream mode: the window kernel's chunk pipeline without the window.  Every
// particle's eight weights go straight to the 64-bit accumulator as L2
// reductions (no return).  Lanes hold consecutive particles; where lane l + 1's
// particle lies in the next z cell of lane l's (x, y) cell column (consecutive
// particles of a lattice, or of any order that runs along z), lane l + 1 adds
// lane l's four upper-z weights to its own four lower-z weights (one shuffle
// each) and lane l skips those four reductions, so each such cell takes one
// reduction for both.  The lower-z reductions of a warp cover consecutive
// cells.  One barrier per chunk; the L2 holds the few x-planes that the
// resident chunks touch.
// Accumulator element of cell (x, y, z): 32-bit arithmetic where the grid has
// fewer than 2^32 elements (WIDE = false), else 64-bit.
template <bool WIDE>
struct CellIndex {
    typedef typename std::conditional<WIDE, int64_t, uint32_t>::type T;
};

template <bool VARMASS, bool CORNER, bool WIDE>
__global__ void __launch_bounds__(kWinThreads, 1)
    k_stream_deposit(WinParams p, DeviceStatus *st, acc_t *__restrict__ acc)
{
    extern __shared__ __align__(128) unsigned char win_smem[];
    float *pbuf = reinterpret_cast<float *>(win_smem);  // [2][chunk * 3]
    float *mbuf = pbuf + 6 * p.chunk;                   // [2][chunk] (VARMASS)
    __shared__ __align__(8) unsigned long long bar[2];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();

    store_host_prep(p, st);
    const int fxs = p.host_prep ? p.fx_shift : st->fx_shift;
    const int emax = 154 - fxs;
    const unsigned ubits = __float_as_uint(p.umass);
    const unsigned umant = (ubits & 0x7fffffu) | 0x800000u;
    const int uef = (int)((ubits >> 23) & 0xffu);
    const bool uneg = (ubits >> 31) != 0u;
    const float mscale = ldexpf(1.f, fxs + 4);

    f2sum alt = {0.f, 0.f};
    unsigned bad = 0, timeouts = 0;
    bool broken = false;  // a wait ran out: plain loads from then on
    const int64_t c0 = blockIdx.x;
    if (threadIdx.x == 0 && c0 < p.nchunks && chunk_by_bulk(p, c0))
        issue_chunk<VARMASS>(p, c0, pbuf, mbuf, &bar[0]);

    int k = 0;
    for (int64_t c = c0; c < p.nchunks; c += gridDim.x, k++) {
        const int buf = k & 1;
        float *P = pbuf + buf * 3 * p.chunk;
        float *M = mbuf + buf * p.chunk;
        const int cnt = (int)min((int64_t)p.chunk, p.n - chunk_first(p, c));
        // The chunk is in place, and every thread is done with the other buffer.
        arrive_chunk<VARMASS>(p, c, cnt, !broken && chunk_by_bulk(p, c), P, M, &bar[buf],
                              (unsigned)(k >> 1) & 1u, broken, timeouts);
        if (threadIdx.x == 0 && !broken && c + gridDim.x < p.nchunks &&
            chunk_by_bulk(p, c + gridDim.x))
            issue_chunk<VARMASS>(p, c + gridDim.x, pbuf + (buf ^ 1) * 3 * p.chunk,
                                 mbuf + (buf ^ 1) * p.chunk, &bar[buf ^ 1]);

        // Same trip count for every lane: the merge shuffles need full warps.
        for (int j0 = 0; j0 < cnt; j0 += blockDim.x) {
            const int j = j0 + threadIdx.x;
            float x = 0.f, y = 0.f, z = 0.f, m = p.umass;
            if (j < cnt) {
                x = P[3 * j];
                y = P[3 * j + 1];
                z = P[3 * j + 2];
                if (VARMASS)
                    m = M[j];
            }
            // The products split_q28 forms first.  Particles at 1 <= |x N/L| <
            // 2^22 cells on every axis (all but those within a cell of the
            // origin, far outside the box, or invalid) take the split without
            // its near-origin step and clamp; the others the general split.
            const float xh = __fmul_rn(x, p.uh), yh = __fmul_rn(y, p.uh), zh = __fmul_rn(z, p.uh);
            bool fast = j < cnt && fabsf(xh) >= 1.f && fabsf(xh) < kFastSplitMax &&
                        fabsf(yh) >= 1.f && fabsf(yh) < kFastSplitMax && fabsf(zh) >= 1.f &&
                        fabsf(zh) < kFastSplitMax;
            if (VARMASS)
                fast = fast && fabsf(m) <= 3.4028235e38f;
            bool valid = fast;
            AxisQ ax, ay, az;
            if (fast) {
                ax = split_q28_unwrapped(x, xh, p.uh, p.ul);
                ay = split_q28_unwrapped(y, yh, p.uh, p.ul);
                az = split_q28_unwrapped(z, zh, p.uh, p.ul);
                // as unsigned values, so that a negative cell reads as out of range
                if (max((unsigned)ax.cell, max((unsigned)ay.cell, (unsigned)az.cell)) >=
                    (unsigned)p.dims) {
                    ax.cell = wrap_cell(ax.cell, p.dims);
                    ay.cell = wrap_cell(ay.cell, p.dims);
                    az.cell = wrap_cell(az.cell, p.dims);
                }
            } else {
                valid = j < cnt;
                if (valid) {
                    bool ok = fabsf(xh) <= kPosLimit && fabsf(yh) <= kPosLimit &&
                              fabsf(zh) <= kPosLimit;
                    if (VARMASS)
                        ok = ok && fabsf(m) <= 3.4028235e38f;
                    if (!ok) {
                        bad++;
                        valid = false;
                        x = y = z = 0.f;
                    }
                }
                ax = split_q28(x, p.uh, p.ul, p.dims);
                ay = split_q28(y, p.uh, p.ul, p.dims);
                az = split_q28(z, p.uh, p.ul, p.dims);
            }
            unsigned mant = umant;
            int ef = uef;
            bool neg = uneg;
            if (VARMASS) {
                const unsigned mb = __float_as_uint(m);
                ef = (int)((mb >> 23) & 0xffu);
                mant = (mb & 0x7fffffu) | 0x800000u;
                neg = (mb >> 31) != 0u;
            }
            valid = valid && ef != 0;  // zero or subnormal mass deposits nothing
            const int dsh = max(emax - ef, 0);
            if (CORNER && valid) {
                f2sum v = corner_factor_q(ax, ay, az);
                if (VARMASS) {
                    const float mm = m * mscale;
                    const float h = __fmul_rn(v.hi, mm);
                    v = f2sum{h, fmaf(v.hi, mm, -h) + v.lo * mm};
                }
                f2_accumulate(alt, f2_signed(v, ax.cell ^ ay.cell ^ az.cell));
            }
            const uint32_t rx = kFracOne - ax.q, ry = kFracOne - ay.q, rz = kFracOne - az.q;
            const uint32_t p00 = pair_w(rx, ry), p10 = pair_w(ax.q, ry), p01 = pair_w(rx, ay.q),
                           p11 = pair_w(ax.q, ay.q);
            const uint32_t zl = z_mass(rz, mant, VARMASS ? dsh : 0);
            const uint32_t zu = z_mass(az.q, mant, VARMASS ? dsh : 0);
            const uint32_t wu[8] = {corner_w(p00, zl), corner_w(p10, zl), corner_w(p01, zl),
                                    corner_w(p11, zl), corner_w(p00, zu), corner_w(p10, zu),
                                    corner_w(p01, zu), corner_w(p11, zu)};
            // Variable masses carry their sign into the merge; a uniform mass's
            // sign is applied at the reductions.
            int w[8];
#pragma unroll
            for (int q = 0; q < 8; q++)
                w[q] = (VARMASS && neg) ? -(int)wu[q] : (int)wu[q];

            // Accumulator elements of the lower-z corner cells (x, y, z) and the
            // +1 steps, wrapped periodically.
            typedef typename CellIndex<WIDE>::T I;
            const I i000 = (I)ax.cell * (I)p.plane + (I)(ay.cell * p.row + az.cell);
            const I dx = ax.cell + 1 == p.dims ? -(I)(p.dims - 1) * (I)p.plane : (I)p.plane;
            const I dy = (I)(ay.cell + 1 == p.dims ? -(p.dims - 1) * p.row : p.row);
            const I dz = (I)(az.cell + 1 == p.dims ? -(p.dims - 1) : 1);

            // Neighbour merge: lane l + 1 takes lane l's upper-z weights when its
            // lower-z cell is lane l's upper-z cell (same x, y cells: the element
            // index fixes all three).  Invalid lanes hold two distinct
            // sentinels that no element index equals.
            const I lower = valid ? i000 : ~(I)0;
            const I upper = valid ? i000 + dz : ~(I)0 - 1;
            const I upper_prev = __shfl_up_sync(0xffffffffu, upper, 1);
            const I lower_next = __shfl_down_sync(0xffffffffu, lower, 1);
            const bool take = lane > 0 && upper_prev == lower;
            const bool give = lane < 31 && lower_next == upper;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int up = __shfl_up_sync(0xffffffffu, w[4 + q], 1);
                w[q] += take ? up : 0;
            }
            if (valid) {
                const I i100 = i000 + dx, i010 = i000 + dy, i110 = i100 + dy;
                if (!VARMASS && !uneg) {  // positive uniform mass: no sign extension
                    atomicAdd(acc + i000, (acc_t)(unsigned)w[0]);
                    atomicAdd(acc + i100, (acc_t)(unsigned)w[1]);
                    atomicAdd(acc + i010, (acc_t)(unsigned)w[2]);
                    atomicAdd(acc + i110, (acc_t)(unsigned)w[3]);
                    if (!give) {
                        atomicAdd(acc + (i000 + dz), (acc_t)(unsigned)w[4]);
                        atomicAdd(acc + (i100 + dz), (acc_t)(unsigned)w[5]);
                        atomicAdd(acc + (i010 + dz), (acc_t)(unsigned)w[6]);
                        atomicAdd(acc + (i110 + dz), (acc_t)(unsigned)w[7]);
                    }
                } else {
                    const long long sg = (!VARMASS && uneg) ? -1 : 1;
                    atomicAdd(acc + i000, (acc_t)(sg * w[0]));
                    atomicAdd(acc + i100, (acc_t)(sg * w[1]));
                    atomicAdd(acc + i010, (acc_t)(sg * w[2]));
                    atomicAdd(acc + i110, (acc_t)(sg * w[3]));
                    if (!give) {
                        atomicAdd(acc + (i000 + dz), (acc_t)(sg * w[4]));
                        atomicAdd(acc + (i100 + dz), (acc_t)(sg * w[5]));
                        atomicAdd(acc + (i010 + dz), (acc_t)(sg * w[6]));
                        atomicAdd(acc + (i110 + dz), (acc_t)(sg * w[7]));
                    }
                }
            }
        }
    }
    report_block<VARMASS, CORNER>(p, st, alt, bad, timeouts, mscale);
}

// Per-CTA FP64 mass partials (Kahan in FP32 first) and the max |mass|.
__global__ void __launch_bounds__(256)
    k_mass_reduce(const float *__restrict__ masses, int64_t n, double *__restrict__ mass_part,
                  DeviceStatus *st)
{
    float s = 0.f, cmp = 0.f, mx = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float m = __ldg(masses + i);
        if (!isfinite(m))
            continue;
        const float y = m - cmp;
        const float t = s + y;
        cmp = (t - s) - y;
        s = t;
        mx = fmaxf(mx, fabsf(m));
    }
    __shared__ double sh[8];
    __shared__ float shm[8];
    double v = warp_sum_d((double)s - (double)cmp);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) {
        sh[threadIdx.x >> 5] = v;
        shm[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t += sh[w];
            m = fmaxf(m, shm[w]);
        }
        mass_part[blockIdx.x] = t;
        if (m > 0.f)
            atomicMax(&st->max_mass_bits, __float_as_uint(m));
    }
}

// Pass constants for the window engine (one thread), as k_sort_scan forms
// them for the sorted engine: pass mass, fixed-point shift s (the largest |mass|
// maps into [2^27, 2^28) units of 2^-s) and the pass mean in fixed point,
// rounded to 24 significant bits (an empty cell then reads back exactly 0).
// nparts = 0: uniform mass umass; else the sum of nparts partial sums.
__global__ void k_window_prep(const double *__restrict__ mass_part, int nparts, double umass,
                              int64_t n, double inv_cells, double *field_mass, double *field_sub,
                              DeviceStatus *st)
{
    double m = 0.0;
    float mref;
    if (nparts == 0) {
        m = (double)n * umass;
        mref = (float)fabs(umass);
    } else {
        for (int c = 0; c < nparts; c++)
            m += mass_part[c];
        mref = __uint_as_float(st->max_mass_bits);
        st->max_mass_bits = 0u;  // read: zero again for the next pass
    }
    const PassConsts k = pass_consts(m, mref, inv_cells);
    st->pass_mass = k.mass;
    st->fx_shift = k.fx_shift;
    st->mean_fixed = k.mean_fixed;
    *field_mass += k.mass;
    *field_sub += ldexp((double)k.mean_fixed, -k.fx_shift);
}

// Accumulator minus the mean, rounded once to FP32 and stored (clean grid) or
// added to the grid, for every real cell: the same conversion as the sorted
// engine's.  Two cells per thread (rows have even length), four pairs in
// flight; grid-stride loop.  The pair's place in its row is tracked
// incrementally (no 64-bit division): the row's last pair is padding for even
// dims and half padding for odd dims, and padding is never written.
__global__ void __launch_bounds__(256)
    k_window_convert(const acc_t *__restrict__ acc, float *__restrict__ grid, int dims, int row,
                     int64_t npairs, int clean, const DeviceStatus *__restrict__ st)
{
    constexpr int U = 4;
    const long long mean = st->mean_fixed;
    const float inv_scale = ldexpf(1.f, -st->fx_shift);
    const int half_row = row >> 1;
    const int last = (dims - 1) >> 1;  // the pair holding z = dims - 1
    const bool odd = (dims & 1) != 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int dz = (int)(stride % half_row);
    int zp = (int)(first % half_row);
    for (int64_t k0 = first; k0 < npairs; k0 += U * stride) {
        longlong2 a[U];
        float2 o[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t k = k0 + u * stride;
            if (k < npairs) {
                a[u] = reinterpret_cast<const longlong2 *>(acc)[k];
                o[u] = clean ? make_float2(0.f, 0.f) : reinterpret_cast<const float2 *>(grid)[k];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t k = k0 + u * stride;
            const int zu = zp;
            zp += dz;
            zp -= zp >= half_row ? half_row : 0;
            if (k >= npairs || zu > last)
                continue;
            const float2 f = make_float2(o[u].x + i64_to_f32_rn(a[u].x - mean) * inv_scale,
                                         o[u].y + i64_to_f32_rn(a[u].y - mean) * inv_scale);
            if (zu < last || !odd)
                reinterpret_cast<float2 *>(grid)[k] = f;
            else
                grid[2 * k] = f.x;
        }
    }
}

__global__ void k_window_finish(DeviceStatus *__restrict__ st, double *field_corner)
{
    *field_corner += ldexp((double)st->alt_sum, -(st->fx_shift + 4));
    st->alt_sum = 0;  // zero for the next pass
}

// Probe: for up to `samples` evenly spread chunks, the window volume in cells
// (the box k_window_deposit's pass A computes for that chunk).
__global__ void __launch_bounds__(256)
    k_window_probe(WinParams p, int samples, long long *__restrict__ vol_out)
{
    __shared__ int sh_mm[6][32];
    __shared__ int sh_box[8];
    const int64_t c = (int64_t)blockIdx.x * p.nchunks / samples;
    const float *P = p.pos + 3 * chunk_first(p, c);
    const int cnt = (int)min((int64_t)p.chunk, p.n - chunk_first(p, c));
    const float ref[3] = {ref_cell(p, P[0]), ref_cell(p, P[1]), ref_cell(p, P[2])};
    float fmn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, fmx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
        float f[3];
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            f[a] = fmaf(P[3 * j + a], p.uh, -ref[a]);
            ok = ok && fabsf(f[a]) <= kPosLimit;
        }
        if (!ok)
            continue;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float w = fmaf(-p.fdims, rintf(f[a] * p.inv_dims), f[a]);
            fmn[a] = fminf(fmn[a], w);
            fmx[a] = fmaxf(fmx[a], w);
        }
    }
    const WinBox box = window_box(fmn, fmx, ref, p, sh_mm, sh_box);
    if (threadIdx.x == 0)
        vol_out[blockIdx.x] = (long long)box.ext[0] * box.ext[1] * box.ext[2];
}

// Probe of the stream mode: over `samples` evenly spread runs of 256
// consecutive particles, how many neighbour pairs within a warp meet the
// stream kernel's merge condition (out[0]) out of all such pairs (out[1]).
__global__ void __launch_bounds__(256)
    k_stream_probe(WinParams p, int samples, unsigned long long *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int64_t j = (((int64_t)blockIdx.x * (p.n - 256) / max(samples - 1, 1)) & ~(int64_t)31) +
                      threadIdx.x;  // warp-aligned like the kernel's lanes
    bool valid = j < p.n;
    float x = 0.f, y = 0.f, z = 0.f;
    if (valid) {
        x = p.pos[3 * j];
        y = p.pos[3 * j + 1];
        z = p.pos[3 * j + 2];
        valid = fabsf(x * p.uh) <= kPosLimit && fabsf(y * p.uh) <= kPosLimit &&
                fabsf(z * p.uh) <= kPosLimit;
        if (!valid)
            x = y = z = 0.f;
    }
    const AxisQ ax = split_q28(x, p.uh, p.ul, p.dims);
    const AxisQ ay = split_q28(y, p.uh, p.ul, p.dims);
    const AxisQ az = split_q28(z, p.uh, p.ul, p.dims);
    const int z1 = az.cell + 1 == p.dims ? 0 : az.cell + 1;
    const int key = valid ? ax.cell * p.dims + ay.cell : -1 - lane;
    const int key_next = __shfl_down_sync(0xffffffffu, key, 1);
    const int z_next = __shfl_down_sync(0xffffffffu, az.cell, 1);
    const bool pair = lane < 31 && j + 1 < p.n;
    const unsigned merged = __popc(__ballot_sync(0xffffffffu, pair && key_next == key && z_next == z1));
    const unsigned pairs = __popc(__ballot_sync(0xffffffffu, pair));
    if (lane == 0) {
        atomicAdd(out, (unsigned long long)merged);
        atomicAdd(out + 1, (unsigned long long)pairs);
    }
}

WinParams make_win_params(const DepositGeom &g, const DepositArgs &a, int chunk)
{
    WinParams p;
    const bool var = a.masses != nullptr;
    p.pos = a.pos;
    p.masses = a.masses;
    p.n = a.n;
    p.chunk = chunk;
    p.nchunks = (a.n + chunk - 1) / chunk;
    p.win_off = chunk * (var ? 32 : 24);
    p.cap = window_cap_cells(chunk, var);
    p.dims = g.grid.dims;
    p.fdims = (float)g.grid.dims;
    p.inv_dims = 1.f / (float)g.grid.dims;
    p.uh = g.units_hi;
    p.ul = g.units_lo;
    p.umass = a.mass;
    p.plane = g.grid.plane;
    p.row = g.grid.row;
    p.corner = (g.grid.dims % 2 == 0) ? 1 : 0;
    // Bulk copies only from device memory; pinned host memory is read in place
    // by plain loads (the transfer over the host link is the bound there).
    p.bulk = (!a.host_mapped && (uintptr_t)a.pos % 16 == 0 &&
              (!var || (uintptr_t)a.masses % 16 == 0))
                 ? 1
                 : 0;
    p.skip_chunk = a.skip_chunk;
    p.skip_wait = a.skip_wait;
    p.host_prep = 0;
    p.fx_shift = 0;
    p.pass_mass = 0.0;
    p.mean_fixed = 0;
    p.field_mass = p.field_sub = nullptr;
    return p;
}

}  // namespace

int window_cap_cells(int chunk, bool variable_masses)
{
    return (kWinSmemBytes - chunk * (variable_masses ? 32 : 24)) / 4;
}

cudaError_t window_probe(const DepositGeom &g, const DepositArgs &a, int chunk,
                         long long *vol_dev, int samples, cudaStream_t stream, int64_t *launches)
{
    const WinParams p = make_win_params(g, a, chunk);
    const int s = (int)std::min<int64_t>(samples, p.nchunks);
    k_window_probe<<<s, 256, 0, stream>>>(p, s, vol_dev);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t stream_probe(const DepositGeom &g, const DepositArgs &a,
                         unsigned long long *out_dev, int samples, cudaStream_t stream,
                         int64_t *launches)
{
    const WinParams p = make_win_params(g, a, kStreamChunk);
    cudaError_t err = cudaMemsetAsync(out_dev, 0, 2 * sizeof(unsigned long long), stream);
    if (err != cudaSuccess)
        return err;
    if (a.n >= 256) {
        k_stream_probe<<<samples, 256, 0, stream>>>(p, samples, out_dev);
        (*launches)++;
    }
    return cudaGetLastError();
}

cudaError_t window_convert(const GridGeom &g, const unsigned long long *acc, float *grid,
                           bool clean, const DeviceStatus *dstat, int num_sms,
                           cudaStream_t stream, int64_t *launches)
{
    k_window_convert<<<num_sms * 8, 256, 0, stream>>>(acc, grid, g.dims, g.row, g.nfloat / 2,
                                                      clean ? 1 : 0, dstat);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t deposit_window_pass(const DepositGeom &g, const DepositArgs &a, int chunk,
                                bool stream_mode, double *mass_part, int mass_ctas,
                                unsigned long long *acc, size_t clear_bytes, bool defer_convert,
                                int num_sms,
                                DeviceStatus *dstat, cudaStream_t stream, int64_t *launches,
                                StageHook hook, void *hook_user)
{
    auto mark = [&](const char *name) {
        (*launches)++;
        if (hook)
            hook(hook_user, name);
    };
    cudaError_t err;
    // (max_mass_bits and alt_sum are zero here: the pass that used them last
    // zeroed them, in k_window_prep / k_sort_scan and the finishing kernels)
    const double n3 = (double)g.grid.dims * g.grid.dims * g.grid.dims;
    WinParams p = make_win_params(g, a, chunk);
    if (a.masses) {
        k_mass_reduce<<<mass_ctas, 256, 0, stream>>>(a.masses, a.n, mass_part, dstat);
        mark("win_mass");
    }
    if (a.masses || p.nchunks == 0) {
        k_window_prep<<<1, 1, 0, stream>>>(mass_part, a.masses ? mass_ctas : 0, (double)a.mass,
                                           a.n, 1.0 / n3, a.field_mass, a.field_sub, dstat);
        mark("win_prep");
    } else {
        // a uniform mass: the constants need nothing from the device, and the
        // deposit kernel stores them (one launch fewer per pass)
        const double umass = (double)a.mass;
        const PassConsts k = pass_consts((double)a.n * umass, (float)fabs(umass), 1.0 / n3);
        p.host_prep = 1;
        p.fx_shift = k.fx_shift;
        p.pass_mass = k.mass;
        p.mean_fixed = k.mean_fixed;
        p.field_mass = a.field_mass;
        p.field_sub = a.field_sub;
    }
    if (clear_bytes) {
        clear_bytes = std::min(clear_bytes, sizeof(acc_t) * (size_t)g.grid.nfloat);
        if ((err = cudaMemsetAsync(acc, 0, clear_bytes, stream)) != cudaSuccess)
            return err;
        mark("win_clear");
    }
    if (p.nchunks > 0) {
        const unsigned ctas = (unsigned)std::min<int64_t>(p.nchunks, num_sms);
        // stream mode: the two chunk buffers only
        const int smem = stream_mode ? p.win_off : p.win_off + 4 * p.cap;
        auto kern = a.masses ? (p.corner ? k_window_deposit<true, true> : k_window_deposit<true, false>)
                             : (p.corner ? k_window_deposit<false, true> : k_window_deposit<false, false>);
        // 32-bit element indices where every index and both sentinels fit.  The
        // environment variable GENPK_WIDE_INDEX=1 forces the 64-bit variant on any grid
        // (a test hook: that variant otherwise runs only from N = 1626 up).
        static const bool force_wide = [] {
            const char *e = std::getenv("GENPK_WIDE_INDEX");
            return e && e[0] == '1';
        }();
        if (stream_mode && !force_wide && g.grid.nfloat < ((int64_t)1 << 32) - 2)
            kern = a.masses ? (p.corner ? k_stream_deposit<true, true, false>
                                        : k_stream_deposit<true, false, false>)
                            : (p.corner ? k_stream_deposit<false, true, false>
                                        : k_stream_deposit<false, false, false>);
        else if (stream_mode)
            kern = a.masses ? (p.corner ? k_stream_deposit<true, true, true>
                                        : k_stream_deposit<true, false, true>)
                            : (p.corner ? k_stream_deposit<false, true, true>
                                        : k_stream_deposit<false, false, true>);
        if ((err = ensure_dynamic_smem(kern, (size_t)smem)) != cudaSuccess)
            return err;
        kern<<<ctas, kWinThreads, smem, stream>>>(p, dstat, acc);
        mark(stream_mode ? "stream_deposit" : "win_deposit");
        if ((err = cudaGetLastError()) != cudaSuccess)
            return err;
    }
    if (!defer_convert) {
        k_window_convert<<<num_sms * 8, 256, 0, stream>>>(acc, a.grid, g.grid.dims, g.grid.row,
                                                          g.grid.nfloat / 2, a.clean ? 1 : 0,
                                                          dstat);
        mark("win_convert");
        if ((err = cudaGetLastError()) != cudaSuccess)
            return err;
    }
    k_window_finish<<<1, 1, 0, stream>>>(dstat, a.field_corner);
    (*launches)++;
    return cudaGetLastError();
}


}  // namespace genpk
