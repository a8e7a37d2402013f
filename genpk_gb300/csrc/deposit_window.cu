// deposit_window.cu -- CIC deposit for spatially coherent particle order.
//
// N-body snapshots usually store particles in a spatially coherent order:
// initial-condition lattice order (the Zel'dovich sets used here), or the
// Peano-Hilbert order of a simulation's domain decomposition.  Then every
// contiguous run of a few thousand particles occupies a small region of the
// grid, and the tile sort in deposit.cu is unnecessary work.  This engine:
//
//   k_window_deposit  one CTA per chunk of `chunk` consecutive particles.
//     pass A  reads the chunk and finds the periodic bounding box of its cells
//             (cells from a plain FP32 product, which is one cell off for a few
//             positions next to a cell face: pass B sends those, if they fall
//             outside the box, down the global path); an axis the chunk spans
//             completely is taken whole, with wrap-around.
//     pass B  re-reads the chunk (from L2) and splits every position exactly
//             (split_axis).  If the box fits the shared window the eight CIC
//             weights go to it with shared FP32 atomics, and the window's
//             non-zero cells are then flushed to the grid row by row with
//             coalesced global atomic adds; otherwise every corner takes a
//             global atomic add.  Pass B also sums the chunk's share of the
//             exact corner mode (see deposit.cu).
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

__device__ __forceinline__ bool pos_ok(const WinParams &p, float x, float y, float z)
{
    if (!finite3(x, y, z))
        return false;
    const float lim = 1.0e9f;
    return !(fabsf(x * p.uh) > lim || fabsf(y * p.uh) > lim || fabsf(z * p.uh) > lim);
}

// Cell from a plain FP32 product: exact or one cell off.
__device__ __forceinline__ int approx_cell(float x, float uh, int dims)
{
    int c = (int)floorf(x * uh);
    if ((unsigned)c >= (unsigned)dims) {
        c %= dims;
        if (c < 0)
            c += dims;
    }
    return c;
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

__device__ __forceinline__ int wrap_once(int v, int n)
{
    return v < 0 ? v + n : (v >= n ? v - n : v);
}

// Periodic bounding box of this thread block's approximate cell offsets:
// reduce (lo, hi) per axis and add one cell for the CIC corner.
__device__ __forceinline__ void block_box(int omin[3], int omax[3], const int ref[3], int dims,
                                          int cap, int (*sh_min)[32], int (*sh_max)[32],
                                          int *sh_box)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        omin[a] = (int)__reduce_min_sync(0xffffffffu, (unsigned)(omin[a] + (1 << 30))) - (1 << 30);
        omax[a] = (int)__reduce_max_sync(0xffffffffu, (unsigned)(omax[a] + (1 << 30))) - (1 << 30);
        if (lane == 0) {
            sh_min[a][wid] = omin[a];
            sh_max[a][wid] = omax[a];
        }
    }
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
            } else if (hi - lo + 2 >= dims) {  // the whole axis, wrapping
                span = dims;
                origin = 0;
            } else {  // +1 for the CIC corner
                span = hi - lo + 2;
                origin = wrap_once(ref[a] + lo, dims);
            }
            sh_box[a] = origin;
            sh_box[3 + a] = span;
            vol *= span;
        }
        sh_box[6] = vol <= cap ? 1 : 0;
    }
    __syncthreads();
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
        const float x = p.pos[3 * b], y = p.pos[3 * b + 1], z = p.pos[3 * b + 2];
        const bool ok = pos_ok(p, x, y, z);
        sh_ref[0] = ok ? approx_cell(x, p.uh, p.dims) : 0;
        sh_ref[1] = ok ? approx_cell(y, p.uh, p.dims) : 0;
        sh_ref[2] = ok ? approx_cell(z, p.uh, p.dims) : 0;
    }
    __syncthreads();
    const int ref[3] = {sh_ref[0], sh_ref[1], sh_ref[2]};

    // Pass A: bounding box of the approximate cells.
    int omin[3] = {1 << 30, 1 << 30, 1 << 30}, omax[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float v[3] = {__ldg(p.pos + 3 * i), __ldg(p.pos + 3 * i + 1),
                            __ldg(p.pos + 3 * i + 2)};
        if (!pos_ok(p, v[0], v[1], v[2]))
            continue;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int o = periodic_offset(approx_cell(v[a], p.uh, p.dims), ref[a], p.dims);
            omin[a] = min(omin[a], o);
            omax[a] = max(omax[a], o);
        }
    }
    block_box(omin, omax, ref, p.dims, p.cap, sh_min, sh_max, sh_box);
    const int org[3] = {sh_box[0], sh_box[1], sh_box[2]};
    const int span[3] = {sh_box[3], sh_box[4], sh_box[5]};
    const bool use_window = sh_box[6] != 0;
    const int sz = span[2], syz = span[1] * span[2];
    if (use_window) {
        const int vol = span[0] * syz;
        for (int i = threadIdx.x; i < vol; i += blockDim.x)
            win[i] = 0.f;
        __syncthreads();
    }

    // Pass B: exact split, weights, corner-mode share.
    const float mscale = ldexpf(1.f, st->fx_shift + 4);
    f2sum alt = {0.f, 0.f};
    unsigned bad = 0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float x = __ldg(p.pos + 3 * i), y = __ldg(p.pos + 3 * i + 1),
                    z = __ldg(p.pos + 3 * i + 2);
        const float m = VARMASS ? __ldg(p.masses + i) : p.umass;
        if (!pos_ok(p, x, y, z) || !isfinite(m)) {
            bad++;
            continue;
        }
        const AxisSplit ax = split_axis(x, p.uh, p.ul, p.dims);
        const AxisSplit ay = split_axis(y, p.uh, p.ul, p.dims);
        const AxisSplit az = split_axis(z, p.uh, p.ul, p.dims);
        if (p.corner) {
            f2sum v = corner_factor(ax, ay, az);
            if (VARMASS) {
                const float mm = m * mscale;
                const float h = __fmul_rn(v.hi, mm);
                v = f2sum{h, fmaf(v.hi, mm, -h) + v.lo * mm};
            }
            if ((ax.cell + ay.cell + az.cell) & 1)
                v = f2sum{-v.hi, -v.lo};
            alt = f2_add2(alt, v);
        }
        const float tx = 1.f - ax.frac, ty = 1.f - ay.frac, tz = 1.f - az.frac;
        // Weight order follows fieldize.cpp:77-84: ((m*wx)*wy)*wz.
        const float mtx = m * tx, mdx = m * ax.frac;
        const float a00 = mtx * ty, a10 = mdx * ty, a01 = mtx * ay.frac, a11 = mdx * ay.frac;
        int w0[3], w1[3];
        bool inwin = use_window;
        if (use_window) {
            const int c[3] = {ax.cell, ay.cell, az.cell};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                int o = c[a] - org[a];
                if (o < 0)
                    o += p.dims;
                w0[a] = o;
                if (span[a] == p.dims) {
                    // whole (wrapping) axis: the +1 corner wraps inside the window
                    w1[a] = o + 1 == p.dims ? 0 : o + 1;
                } else {
                    w1[a] = o + 1;
                    // The box came from approximate cells (a plain FP32 product
                    // is one cell off for ~1e-4 of positions near a cell face):
                    // a particle whose exact cell falls outside the window takes
                    // the global path.
                    inwin = inwin && (o + 1 < span[a]);
                }
            }
        }
        if (inwin) {
            const int x0 = w0[0] * syz, x1 = w1[0] * syz, y0 = w0[1] * sz, y1 = w1[1] * sz;
            atomicAdd(&win[x0 + y0 + w0[2]], a00 * tz);
            atomicAdd(&win[x1 + y0 + w0[2]], a10 * tz);
            atomicAdd(&win[x0 + y1 + w0[2]], a01 * tz);
            atomicAdd(&win[x1 + y1 + w0[2]], a11 * tz);
            atomicAdd(&win[x0 + y0 + w1[2]], a00 * az.frac);
            atomicAdd(&win[x1 + y0 + w1[2]], a10 * az.frac);
            atomicAdd(&win[x0 + y1 + w1[2]], a01 * az.frac);
            atomicAdd(&win[x1 + y1 + w1[2]], a11 * az.frac);
        } else {
            const int cx = ax.cell, cy = ay.cell, cz = az.cell;
            const int hx = cx + 1 == p.dims ? 0 : cx + 1, hy = cy + 1 == p.dims ? 0 : cy + 1,
                      hz = cz + 1 == p.dims ? 0 : cz + 1;
            atomicAdd(grid + cell_index(p.plane, p.row, cx, cy, cz), a00 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, hx, cy, cz), a10 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, cx, hy, cz), a01 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, hx, hy, cz), a11 * tz);
            atomicAdd(grid + cell_index(p.plane, p.row, cx, cy, hz), a00 * az.frac);
            atomicAdd(grid + cell_index(p.plane, p.row, hx, cy, hz), a10 * az.frac);
            atomicAdd(grid + cell_index(p.plane, p.row, cx, hy, hz), a01 * az.frac);
            atomicAdd(grid + cell_index(p.plane, p.row, hx, hy, hz), a11 * az.frac);
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
            if (!VARMASS) {  // the uniform mass was factored out of the sum
                const float mm = p.umass * mscale;
                const float h = __fmul_rn(alt.hi, mm);
                alt = f2sum{h, fmaf(alt.hi, mm, -h) + alt.lo * mm};
            }
            const long long w = __float2ll_rn(alt.hi) + __float2ll_rn(alt.lo);
            if (w != 0)
                atomicAdd((unsigned long long *)&st->alt_sum, (unsigned long long)w);
        }
    }
    bad = __reduce_add_sync(0xffffffffu, bad);
    if (lane == 0 && bad)
        atomicAdd(&st->bad_particles, (unsigned long long)bad);
    if (!use_window)
        return;
    __syncthreads();
    // Flush: one warp per window row (one division per row), lanes along z.
    // Whole rows (the window spans all of z) go out as 16-byte vector atomics
    // from the first 16-byte-aligned cell on; everything else cell by cell.
    const int nrows = span[0] * span[1];
    const int nwarps = blockDim.x >> 5;
    const bool whole_z = span[2] == p.dims && p.dims >= 8;
    for (int r = wid; r < nrows; r += nwarps) {
        const int wx = r / span[1];
        const int wy = r - wx * span[1];
        const int gx = wrap_once(org[0] + wx, p.dims), gy = wrap_once(org[1] + wy, p.dims);
        float *grow = grid + (size_t)gx * (size_t)p.plane + (size_t)gy * (size_t)p.row;
        const float *wrow = win + (size_t)r * sz;
        if (whole_z) {
            // [zv, zend) as float4; the (at most 3 + 3) cells either side scalar
            const int zv = (int)(((16u - ((unsigned)(uintptr_t)grow & 15u)) & 15u) >> 2);
            const int zend = zv + ((p.dims - zv) & ~3);
            for (int z = zv + 4 * lane; z < zend; z += 128) {
                const float4 v = make_float4(wrow[z], wrow[z + 1], wrow[z + 2], wrow[z + 3]);
                if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f)
                    atomicAdd((float4 *)(grow + z), v);
            }
            const int ze = lane < zv ? lane : zend + lane - zv;
            if (ze < p.dims && (lane < zv || lane - zv < p.dims - zend)) {
                const float v = wrow[ze];
                if (v != 0.f)
                    atomicAdd(grow + ze, v);
            }
            continue;
        }
        for (int z = lane; z < sz; z += 32) {
            const float v = wrow[z];
            if (v != 0.f) {
                int gz = org[2] + z;
                gz -= gz >= p.dims ? p.dims : 0;
                atomicAdd(grow + gz, v);
            }
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
// shift (used by the corner sum), the mean as a float (so -mean is exact in
// FP32 and read-back adds back exactly what was subtracted), and the running
// totals of the grid.
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

// Probe: for up to `samples` evenly spread chunks, the box volume in cells
// (computed as pass A of k_window_deposit does).
__global__ void __launch_bounds__(256)
    k_window_probe(WinParams p, int samples, int64_t nchunks, long long *__restrict__ vol_out)
{
    const int s = blockIdx.x;
    const int64_t chunk_id = (int64_t)s * nchunks / samples;
    const int64_t b = chunk_id * p.chunk;
    const int64_t e = min(p.n, b + (int64_t)p.chunk);
    __shared__ int sh_ref[3];
    __shared__ int sh_min[3][32], sh_max[3][32];
    __shared__ int sh_box[7];
    if (threadIdx.x == 0) {
        const float x = p.pos[3 * b], y = p.pos[3 * b + 1], z = p.pos[3 * b + 2];
        const bool ok = pos_ok(p, x, y, z);
        sh_ref[0] = ok ? approx_cell(x, p.uh, p.dims) : 0;
        sh_ref[1] = ok ? approx_cell(y, p.uh, p.dims) : 0;
        sh_ref[2] = ok ? approx_cell(z, p.uh, p.dims) : 0;
    }
    __syncthreads();
    const int ref[3] = {sh_ref[0], sh_ref[1], sh_ref[2]};
    int omin[3] = {1 << 30, 1 << 30, 1 << 30}, omax[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float v[3] = {p.pos[3 * i], p.pos[3 * i + 1], p.pos[3 * i + 2]};
        if (!pos_ok(p, v[0], v[1], v[2]))
            continue;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int o = periodic_offset(approx_cell(v[a], p.uh, p.dims), ref[a], p.dims);
            omin[a] = min(omin[a], o);
            omax[a] = max(omax[a], o);
        }
    }
    block_box(omin, omax, ref, p.dims, p.cap, sh_min, sh_max, sh_box);
    if (threadIdx.x == 0)
        vol_out[s] = (long long)sh_box[3] * sh_box[4] * sh_box[5];
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
