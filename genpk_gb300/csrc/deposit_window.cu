// deposit_window.cu -- CIC deposit for spatially coherent particle order.
//
// N-body snapshots usually store particles in a spatially coherent order:
// initial-condition lattice order (the Zel'dovich sets used here), or the
// Peano-Hilbert order of a simulation's domain decomposition.  Then every
// contiguous run of a few thousand particles occupies a small region of the
// grid, and the tile sort in deposit.cu is unnecessary work.  This engine:
//
//   k_window_deposit  one CTA per chunk of `chunk` consecutive particles.
//     pass A  reads the chunk, finds the periodic bounding box of its cells
//             relative to the chunk's first particle (an axis the chunk spans
//             completely is taken whole, with wrap-around), and adds the
//             chunk's share of the exact corner mode (see deposit.cu).
//     pass B  if the box (+1 for the CIC corner) fits the shared window, it
//             re-reads the chunk (from L2), accumulates the eight CIC weights
//             with shared FP32 atomics and flushes the window's non-zero cells
//             to the grid with coalesced global atomic adds.  Otherwise every
//             corner goes to the grid with a global atomic add.
//
// The grid is first filled with -mean (k_grid_fill / k_grid_add), the pass mean
// computed in k_window_prep, so the result is mean-subtracted like the sorted
// engine's.  FP32 atomics make the low bits depend on summation order; the
// sorted engine (deposit.cu) is the exact, bit-reproducible alternative.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace genpk {
namespace {

constexpr int kWinThreads = 1024;

struct WinParams {
    const float *pos;
    const float *masses;
    int64_t n;
    int chunk;
    int cap;     // window capacity in cells
    int dims;
    float uh, ul;
    float umass;
    int64_t plane;
    int row;
    int corner;  // accumulate the exact (N/2,N/2,N/2) mode (even grids)
};

__device__ __forceinline__ bool win_cell(const WinParams &p, float x, float y, float z, float m,
                                         int c[3], float d[3])
{
    if (!finite3(x, y, z) || !isfinite(m))
        return false;
    const float lim = 1.0e9f;
    if (fabsf(x * p.uh) > lim || fabsf(y * p.uh) > lim || fabsf(z * p.uh) > lim)
        return false;
    split_cell(x, p.uh, p.ul, p.dims, c[0], d[0]);
    split_cell(y, p.uh, p.ul, p.dims, c[1], d[1]);
    split_cell(z, p.uh, p.ul, p.dims, c[2], d[2]);
    return true;
}

// Signed offset of cell c from ref on a periodic axis, in [-N/2, N/2).
__device__ __forceinline__ int periodic_offset(int c, int ref, int n)
{
    int o = c - ref;
    if (o < -(n >> 1))
        o += n;
    if (o >= n - (n >> 1))
        o -= n;
    return o;
}

template <bool VARMASS>
__global__ void __launch_bounds__(kWinThreads)
    k_window_deposit(WinParams p, DeviceStatus *st, float *__restrict__ grid)
{
    extern __shared__ float win[];
    __shared__ int sh_ref[3];
    __shared__ int sh_min[3][32], sh_max[3][32];
    __shared__ int sh_box[7];  // origin[3], span[3], use_window
    const int64_t b = (int64_t)blockIdx.x * p.chunk;
    const int64_t e = min(p.n, b + (int64_t)p.chunk);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        int c[3] = {0, 0, 0};
        float d[3];
        const float m0 = VARMASS ? p.masses[b] : 0.f;
        if (!win_cell(p, p.pos[3 * b], p.pos[3 * b + 1], p.pos[3 * b + 2], m0, c, d))
            c[0] = c[1] = c[2] = 0;
        sh_ref[0] = c[0];
        sh_ref[1] = c[1];
        sh_ref[2] = c[2];
    }
    __syncthreads();
    const int ref[3] = {sh_ref[0], sh_ref[1], sh_ref[2]};

    // Pass A: periodic bounding box, bad particles, exact corner share.
    int omin[3] = {1 << 30, 1 << 30, 1 << 30}, omax[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    unsigned bad = 0;
    const float mscale = ldexpf(1.f, st->fx_shift + 4);
    f2sum alt = {0.f, 0.f};
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float x = __ldg(p.pos + 3 * i), y = __ldg(p.pos + 3 * i + 1),
                    z = __ldg(p.pos + 3 * i + 2);
        const float m = VARMASS ? __ldg(p.masses + i) : p.umass;
        int c[3];
        float d[3];
        if (!win_cell(p, x, y, z, m, c, d)) {
            bad++;
            continue;
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int o = periodic_offset(c[a], ref[a], p.dims);
            omin[a] = min(omin[a], o);
            omax[a] = max(omax[a], o);
        }
        if (p.corner) {
            f2sum u = f2_mul(one_minus_2frac(x, p.uh, p.ul), one_minus_2frac(y, p.uh, p.ul));
            u = f2_mul(u, one_minus_2frac(z, p.uh, p.ul));
            u = f2_mul(u, f2sum{m * mscale, 0.f});
            if ((c[0] + c[1] + c[2]) & 1)
                u = f2sum{-u.hi, -u.lo};
            alt = f2_add2(alt, u);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        omin[a] = __reduce_min_sync(0xffffffffu, (unsigned)(omin[a] + (1 << 30))) - (1 << 30);
        omax[a] = (int)__reduce_max_sync(0xffffffffu, (unsigned)(omax[a] + (1 << 30))) - (1 << 30);
        if (lane == 0) {
            sh_min[a][wid] = omin[a];
            sh_max[a][wid] = omax[a];
        }
    }
    if (p.corner) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const f2sum other = {__shfl_xor_sync(0xffffffffu, alt.hi, o),
                                 __shfl_xor_sync(0xffffffffu, alt.lo, o)};
            alt = f2_add2(alt, other);
        }
        if (lane == 0) {
            const long long w = __float2ll_rn(alt.hi) + __float2ll_rn(alt.lo);
            if (w != 0)
                atomicAdd((unsigned long long *)&st->alt_sum, (unsigned long long)w);
        }
    }
    bad = __reduce_add_sync(0xffffffffu, bad);
    if (lane == 0 && bad)
        atomicAdd(&st->bad_particles, (unsigned long long)bad);
    __syncthreads();
    if (threadIdx.x == 0) {
        long long vol = 1;
        const int nw = blockDim.x >> 5;
        for (int a = 0; a < 3; a++) {
            int lo = 1 << 30, hi = -(1 << 30);
            for (int w = 0; w < nw; w++) {
                lo = min(lo, sh_min[a][w]);
                hi = max(hi, sh_max[a][w]);
            }
            int span, origin;
            if (hi < lo) {  // no valid particle
                span = 1;
                origin = 0;
            } else if (hi - lo + 2 >= p.dims) {  // the whole axis, wrapping
                span = p.dims;
                origin = 0;
            } else {
                span = hi - lo + 2;
                origin = ref[a] + lo;
                origin = origin < 0 ? origin + p.dims : (origin >= p.dims ? origin - p.dims : origin);
            }
            sh_box[a] = origin;
            sh_box[3 + a] = span;
            vol *= span;
        }
        sh_box[6] = vol <= p.cap ? 1 : 0;
    }
    __syncthreads();
    const int org[3] = {sh_box[0], sh_box[1], sh_box[2]};
    const int span[3] = {sh_box[3], sh_box[4], sh_box[5]};
    const bool use_window = sh_box[6] != 0;

    if (use_window) {
        const int vol = span[0] * span[1] * span[2];
        for (int i = threadIdx.x; i < vol; i += blockDim.x)
            win[i] = 0.f;
        __syncthreads();
        const int sz = span[2], syz = span[1] * span[2];
        for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
            const float x = __ldg(p.pos + 3 * i), y = __ldg(p.pos + 3 * i + 1),
                        z = __ldg(p.pos + 3 * i + 2);
            const float m = VARMASS ? __ldg(p.masses + i) : p.umass;
            int c[3];
            float d[3];
            if (!win_cell(p, x, y, z, m, c, d))
                continue;
            int w0[3], w1[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                int o = c[a] - org[a];
                if (o < 0)
                    o += p.dims;
                w0[a] = o;
                // the +1 corner; on a whole (wrapping) axis it wraps inside the window
                w1[a] = (span[a] == p.dims && o + 1 == p.dims) ? 0 : o + 1;
            }
            const float tx = 1.f - d[0], ty = 1.f - d[1], tz = 1.f - d[2];
            // Weight order follows fieldize.cpp:77-84: ((m*wx)*wy)*wz.
            const float mtx = m * tx, mdx = m * d[0];
            const float a00 = mtx * ty, a10 = mdx * ty, a01 = mtx * d[1], a11 = mdx * d[1];
            const int x0 = w0[0] * syz, x1 = w1[0] * syz, y0 = w0[1] * sz, y1 = w1[1] * sz;
            atomicAdd(&win[x0 + y0 + w0[2]], a00 * tz);
            atomicAdd(&win[x1 + y0 + w0[2]], a10 * tz);
            atomicAdd(&win[x0 + y1 + w0[2]], a01 * tz);
            atomicAdd(&win[x1 + y1 + w0[2]], a11 * tz);
            atomicAdd(&win[x0 + y0 + w1[2]], a00 * d[2]);
            atomicAdd(&win[x1 + y0 + w1[2]], a10 * d[2]);
            atomicAdd(&win[x0 + y1 + w1[2]], a01 * d[2]);
            atomicAdd(&win[x1 + y1 + w1[2]], a11 * d[2]);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < vol; i += blockDim.x) {
            const float v = win[i];
            if (v == 0.f)
                continue;
            const int wx = i / syz, wy = (i / sz) % span[1], wz = i % sz;
            int gx = org[0] + wx, gy = org[1] + wy, gz = org[2] + wz;
            gx -= gx >= p.dims ? p.dims : 0;
            gy -= gy >= p.dims ? p.dims : 0;
            gz -= gz >= p.dims ? p.dims : 0;
            atomicAdd(grid + cell_index(p.plane, p.row, gx, gy, gz), v);
        }
    } else {
        for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
            const float x = __ldg(p.pos + 3 * i), y = __ldg(p.pos + 3 * i + 1),
                        z = __ldg(p.pos + 3 * i + 2);
            const float m = VARMASS ? __ldg(p.masses + i) : p.umass;
            int c[3];
            float d[3];
            if (!win_cell(p, x, y, z, m, c, d))
                continue;
            int h[3];
#pragma unroll
            for (int a = 0; a < 3; a++)
                h[a] = c[a] + 1 == p.dims ? 0 : c[a] + 1;
            const float tx = 1.f - d[0], ty = 1.f - d[1], tz = 1.f - d[2];
            const float mtx = m * tx, mdx = m * d[0];
            const float a00 = mtx * ty, a10 = mdx * ty, a01 = mtx * d[1], a11 = mdx * d[1];
            atomicAdd(grid + cell_index(p.plane, p.row, c[0], c[1], c[2]), a00 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, h[0], c[1], c[2]), a10 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, c[0], h[1], c[2]), a01 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, h[0], h[1], c[2]), a11 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, c[0], c[1], h[2]), a00 * d[2]);
            atomicAdd(grid + cell_index(p.plane, p.row, h[0], c[1], h[2]), a10 * d[2]);
            atomicAdd(grid + cell_index(p.plane, p.row, c[0], h[1], h[2]), a01 * d[2]);
            atomicAdd(grid + cell_index(p.plane, p.row, h[0], h[1], h[2]), a11 * d[2]);
        }
    }
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

// Pass constants for the window engine (one thread): pass mass, fixed-point
// shift (used by the corner sum), the mean rounded so that -mean is exact in
// FP32, and the running totals of the grid.
__global__ void k_window_prep(const double *__restrict__ mass_part, int nparts, double umass,
                              int64_t n, double inv_cells, double *field_mass, double *field_sub,
                              DeviceStatus *st)
{
    double m = 0.0;
    float mref;
    if (umass >= 0.0) {
        m = (double)n * umass;
        mref = (float)umass;
    } else {
        for (int c = 0; c < nparts; c++)
            m += mass_part[c];
        mref = __uint_as_float(st->max_mass_bits);
    }
    int s = 0;
    if (mref > 0.f && isfinite(mref))
        s = 27 - ilogbf(mref);
    s = max(-100, min(100, s));
    // mean as a float with 24 significant bits exactly: -mean is exact in FP32
    const float mean32 = (float)(m * inv_cells);
    st->pass_mass = m;
    st->fx_shift = s;
    st->win_mean = mean32;
    *field_mass += m;
    *field_sub += (double)mean32;
}

// grid[i] = -mean for every float (padding included: it is overwritten later).
__global__ void k_grid_fill(float *__restrict__ grid, int64_t nfloat, const DeviceStatus *st)
{
    const float v = -st->win_mean;
    float4 *g4 = (float4 *)grid;
    const int64_t n4 = nfloat >> 2;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
         i += (int64_t)gridDim.x * blockDim.x)
        g4[i] = make_float4(v, v, v, v);
    for (int64_t i = (n4 << 2) + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nfloat;
         i += (int64_t)gridDim.x * blockDim.x)
        grid[i] = v;
}

// grid[real cells] += -mean (accumulating passes).
__global__ void k_grid_add(float *__restrict__ grid, int dims, int row, int64_t ncells_rows,
                           const DeviceStatus *st)
{
    const float v = -st->win_mean;
    const int64_t total = ncells_rows * row;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        if ((int)(i % row) < dims)
            grid[i] += v;
    }
}

__global__ void k_window_finish(const DeviceStatus *__restrict__ st, double *field_corner)
{
    *field_corner += ldexp((double)st->alt_sum, -(st->fx_shift + 4));
}

// Probe: for up to `samples` evenly spread chunks, the box volume in cells.
__global__ void __launch_bounds__(256)
    k_window_probe(WinParams p, int samples, int64_t nchunks, long long *__restrict__ vol_out)
{
    const int s = blockIdx.x;
    const int64_t chunk_id = (int64_t)s * nchunks / samples;
    const int64_t b = chunk_id * p.chunk;
    const int64_t e = min(p.n, b + (int64_t)p.chunk);
    __shared__ int ref[3];
    __shared__ int mn[3][8], mx[3][8];
    if (threadIdx.x == 0) {
        int c[3] = {0, 0, 0};
        float d[3];
        if (!win_cell(p, p.pos[3 * b], p.pos[3 * b + 1], p.pos[3 * b + 2], 0.f, c, d))
            c[0] = c[1] = c[2] = 0;
        ref[0] = c[0];
        ref[1] = c[1];
        ref[2] = c[2];
    }
    __syncthreads();
    int omin[3] = {1 << 30, 1 << 30, 1 << 30}, omax[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        int c[3];
        float d[3];
        if (!win_cell(p, p.pos[3 * i], p.pos[3 * i + 1], p.pos[3 * i + 2], 0.f, c, d))
            continue;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int o = periodic_offset(c[a], ref[a], p.dims);
            omin[a] = min(omin[a], o);
            omax[a] = max(omax[a], o);
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        omin[a] = __reduce_min_sync(0xffffffffu, (unsigned)(omin[a] + (1 << 30))) - (1 << 30);
        omax[a] = (int)__reduce_max_sync(0xffffffffu, (unsigned)(omax[a] + (1 << 30))) - (1 << 30);
        if (lane == 0) {
            mn[a][wid] = omin[a];
            mx[a][wid] = omax[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long vol = 1;
        for (int a = 0; a < 3; a++) {
            int lo = 1 << 30, hi = -(1 << 30);
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                lo = min(lo, mn[a][w]);
                hi = max(hi, mx[a][w]);
            }
            const int span = hi < lo ? 1 : min(hi - lo + 2, p.dims);
            vol *= span;
        }
        vol_out[s] = vol;
    }
}

WinParams make_win_params(const DepositGeom &g, const DepositArgs &a, int chunk, int cap)
{
    WinParams p;
    p.pos = a.pos;
    p.masses = a.masses;
    p.n = a.n;
    p.chunk = chunk;
    p.cap = cap;
    p.dims = g.grid.dims;
    p.uh = g.units_hi;
    p.ul = g.units_lo;
    p.umass = a.mass;
    p.plane = g.grid.plane;
    p.row = g.grid.row;
    p.corner = (g.grid.dims % 2 == 0) ? 1 : 0;
    return p;
}

}  // namespace

// Chunk length: small enough that a lattice-ordered chunk (rows of dims
// particles) covers well under half of the grid along any axis, large enough
// that a window is reused by many particles.
int window_chunk(int dims)
{
    if (dims > 512)
        return 4096;
    const int64_t quarter_plane = (int64_t)dims * dims / 8;
    return (int)std::max<int64_t>(1024, std::min<int64_t>(8192, quarter_plane));
}

cudaError_t window_probe(const DepositGeom &g, const DepositArgs &a, long long *vol_dev,
                         int samples, cudaStream_t stream, int64_t *launches)
{
    const int chunk = window_chunk(g.grid.dims);
    const WinParams p = make_win_params(g, a, chunk, kWindowCapCells);
    const int64_t nchunks = (a.n + chunk - 1) / chunk;
    const int s = (int)std::min<int64_t>(samples, nchunks);
    k_window_probe<<<s, 256, 0, stream>>>(p, s, nchunks, vol_dev);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t deposit_window_pass(const DepositGeom &g, const DepositArgs &a, double *mass_part,
                                int mass_ctas, DeviceStatus *dstat, cudaStream_t stream,
                                int64_t *launches, StageHook hook, void *hook_user)
{
    auto mark = [&](const char *name) {
        (*launches)++;
        if (hook)
            hook(hook_user, name);
    };
    cudaError_t err;
    if ((err = cudaMemsetAsync(&dstat->max_mass_bits, 0, sizeof(unsigned), stream)) != cudaSuccess)
        return err;
    if ((err = cudaMemsetAsync(&dstat->alt_sum, 0, sizeof(long long), stream)) != cudaSuccess)
        return err;
    const double n3 = (double)g.grid.dims * g.grid.dims * g.grid.dims;
    if (a.masses) {
        k_mass_reduce<<<mass_ctas, 256, 0, stream>>>(a.masses, a.n, mass_part, dstat);
        mark("win_mass");
    }
    k_window_prep<<<1, 1, 0, stream>>>(mass_part, mass_ctas, a.masses ? -1.0 : (double)a.mass,
                                       a.n, 1.0 / n3, a.field_mass, a.field_sub, dstat);
    mark("win_prep");
    const int fill_blocks = 152 * 8;
    if (a.clean)
        k_grid_fill<<<fill_blocks, 256, 0, stream>>>(a.grid, g.grid.nfloat, dstat);
    else
        k_grid_add<<<fill_blocks, 256, 0, stream>>>(a.grid, g.grid.dims, g.grid.row,
                                                     (int64_t)g.grid.dims * g.grid.dims, dstat);
    mark("win_fill");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    const int chunk = window_chunk(g.grid.dims);
    const WinParams p = make_win_params(g, a, chunk, kWindowCapCells);
    const int64_t nchunks = (a.n + chunk - 1) / chunk;
    const size_t smem = sizeof(float) * (size_t)kWindowCapCells;
    if (a.masses) {
        if ((err = cudaFuncSetAttribute(k_window_deposit<true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
            return err;
        k_window_deposit<true><<<(unsigned)nchunks, kWinThreads, smem, stream>>>(p, dstat, a.grid);
    } else {
        if ((err = cudaFuncSetAttribute(k_window_deposit<false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
            return err;
        k_window_deposit<false><<<(unsigned)nchunks, kWinThreads, smem, stream>>>(p, dstat,
                                                                                a.grid);
    }
    mark("win_deposit");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    k_window_finish<<<1, 1, 0, stream>>>(dstat, a.field_corner);
    (*launches)++;
    return cudaGetLastError();
}

}  // namespace genpk
