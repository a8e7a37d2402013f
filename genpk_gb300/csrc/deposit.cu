// deposit.cu -- CIC mass assignment (the GPU counterpart of fieldize.cpp:46-113).
//
// One deposit pass over n particles runs five kernels on one stream:
//
//   K1 k_sort_hist      each CTA owns a contiguous particle range; it computes
//                       every particle's cell (two-product split, see
//                       split_cell), counts particles per tile in a shared
//                       histogram and writes that histogram row to scratch.
//                       It also sums variable masses (Kahan, FP32 -> FP64).
//   K2 k_sort_colsum    per tile: total over the CTA rows.
//   K3 k_sort_scan      one CTA: exclusive scan of the tile totals -> tile_start,
//                       and the pass mass (FP64) for the mean subtraction.
//   K4 k_sort_offsets   per tile: turns the histogram rows into each CTA's first
//                       slot in that tile (a column scan).
//   K5 k_sort_scatter   re-reads the range and writes each particle, packed as
//                       tile-local cell + 24-bit fraction per axis (+ mass), to
//                       its slot: a counting sort into tile order.
//   K6 k_tile_deposit   one CTA per tile: accumulates its particles' eight CIC
//                       weights in a (T+1)^3 shared-memory block, stores the
//                       T^3 interior to the grid minus the pass mean (coalesced
//                       rows; a plain store when the grid is freshly zeroed,
//                       read-modify-write otherwise) and the +1 halo faces to
//                       scratch.
//   K7 k_halo_merge     adds every tile's halo faces to the neighbouring cells.
//
// Every grid cell is written by exactly one CTA in K6 and receives halo sums
// in K7, so no grid memset is needed before the first pass and no global
// atomics touch the interior.  Mean subtraction keeps the FP32 r2c accurate:
// each pass removes its own mass / N^3 from every real cell, which changes only
// the (excluded) k = 0 mode.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace genpk {

GridGeom make_grid_geom(int dims)
{
    GridGeom g;
    g.dims = dims;
    g.half = dims / 2;
    g.hc = dims / 2 + 1;
    g.row = 2 * g.hc;
    g.plane = (int64_t)g.row * dims;
    g.nfloat = g.plane * dims;
    return g;
}

namespace {

struct SortParams {
    const float *pos;
    const float *masses;
    int64_t n;
    int64_t chunk;   // particles per sort CTA
    int dims;
    float uh, ul;
    int lx, ly, lz;  // log2 of the tile edges
    int nty, ntz;
    int ntiles;
};

constexpr int kSortThreads = 512;
constexpr int kSortUnroll = 4;

// Cell and tile of one particle; false for a particle that must be skipped.
__device__ __forceinline__ bool particle_cell(const SortParams &p, float x, float y, float z,
                                              int c[3], float d[3], uint32_t &tile)
{
    if (!finite3(x, y, z))
        return false;
    const float lim = 1.0e9f;
    if (fabsf(x * p.uh) > lim || fabsf(y * p.uh) > lim || fabsf(z * p.uh) > lim)
        return false;
    split_cell(x, p.uh, p.ul, p.dims, c[0], d[0]);
    split_cell(y, p.uh, p.ul, p.dims, c[1], d[1]);
    split_cell(z, p.uh, p.ul, p.dims, c[2], d[2]);
    tile = ((uint32_t)(c[0] >> p.lx) * (uint32_t)p.nty + (uint32_t)(c[1] >> p.ly)) *
               (uint32_t)p.ntz +
           (uint32_t)(c[2] >> p.lz);
    return true;
}

__global__ void __launch_bounds__(kSortThreads)
    k_sort_hist(SortParams p, uint32_t *__restrict__ hist, double *__restrict__ mass_part,
                DeviceStatus *st)
{
    extern __shared__ uint32_t sh_hist[];
    __shared__ double sh_mass[kSortThreads / 32];
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
        sh_hist[i] = 0u;
    __syncthreads();

    const int64_t b = (int64_t)blockIdx.x * p.chunk;
    const int64_t e = min(p.n, b + p.chunk);
    const float *__restrict__ pos = p.pos;
    float msum = 0.f, mc = 0.f;
    unsigned bad = 0;
    for (int64_t i0 = b + threadIdx.x; i0 < e; i0 += (int64_t)kSortUnroll * blockDim.x) {
        float v[kSortUnroll][3];
        float m[kSortUnroll];
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++) {
            const int64_t i = i0 + (int64_t)u * blockDim.x;
            if (i < e) {
                v[u][0] = __ldg(pos + 3 * i);
                v[u][1] = __ldg(pos + 3 * i + 1);
                v[u][2] = __ldg(pos + 3 * i + 2);
                m[u] = p.masses ? __ldg(p.masses + i) : 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++) {
            const int64_t i = i0 + (int64_t)u * blockDim.x;
            if (i >= e)
                break;
            int c[3];
            float d[3];
            uint32_t t;
            if (!particle_cell(p, v[u][0], v[u][1], v[u][2], c, d, t) || !isfinite(m[u])) {
                bad++;
                continue;
            }
            atomicAdd(&sh_hist[t], 1u);
            // Kahan-compensated FP32 sum of this thread's masses.
            const float y = m[u] - mc;
            const float s = msum + y;
            mc = (s - msum) - y;
            msum = s;
        }
    }
    __syncthreads();
    uint32_t *row = hist + (size_t)blockIdx.x * p.ntiles;
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
        row[i] = sh_hist[i];

    double md = warp_sum_d((double)msum - (double)mc);
    if ((threadIdx.x & 31) == 0)
        sh_mass[threadIdx.x >> 5] = md;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++)
            s += sh_mass[w];
        mass_part[blockIdx.x] = s;
    }
    if (bad)
        atomicAdd(&st->bad_particles, (unsigned long long)bad);
}

__global__ void k_sort_colsum(const uint32_t *__restrict__ hist, int nsort, int ntiles,
                              uint32_t *__restrict__ totals)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles)
        return;
    uint32_t s = 0;
    for (int c = 0; c < nsort; c++)
        s += hist[(size_t)c * ntiles + t];
    totals[t] = s;
}

constexpr int kScanThreads = 1024;

// Exclusive scan of tile totals (one CTA, chunks of kScanThreads) and the pass
// mass.  uniform_mass >= 0 means every particle weighs uniform_mass.
__global__ void __launch_bounds__(kScanThreads)
    k_sort_scan(const uint32_t *__restrict__ totals, int ntiles, uint32_t *__restrict__ tile_start,
                const double *__restrict__ mass_part, int nsort, double uniform_mass,
                double *field_mass, DeviceStatus *st)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ uint32_t carry;
    __shared__ double sh_m[kScanThreads / 32];
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < ntiles; base += kScanThreads) {
        const int t = base + threadIdx.x;
        const uint32_t v = t < ntiles ? totals[t] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o)
                x += y;
        }
        if (lane == 31)
            warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o)
                    w += y;
            }
            warp_tot[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t before = (wid ? warp_tot[wid - 1] : 0u) + carry;
        if (t < ntiles)
            tile_start[t] = before + x - v;
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1)
            carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        tile_start[ntiles] = carry;

    // Pass mass.
    double m = 0.0;
    if (uniform_mass < 0.0) {
        for (int c = threadIdx.x; c < nsort; c += blockDim.x)
            m += mass_part[c];
        m = warp_sum_d(m);
        if (lane == 0)
            sh_m[wid] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < kScanThreads / 32; w++)
                s += sh_m[w];
            m = s;
        }
    } else {
        m = (double)carry * uniform_mass;
    }
    if (threadIdx.x == 0) {
        st->pass_mass = m;
        *field_mass += m;
    }
}

__global__ void k_sort_offsets(uint32_t *__restrict__ hist, int nsort, int ntiles,
                               const uint32_t *__restrict__ tile_start)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles)
        return;
    uint32_t run = tile_start[t];
    for (int c = 0; c < nsort; c++) {
        const size_t k = (size_t)c * ntiles + t;
        const uint32_t v = hist[k];
        hist[k] = run;
        run += v;
    }
}

// Packed particle: per axis (tile-local cell << 24) | 24-bit fraction; w = mass bits.
template <bool VARMASS>
__global__ void __launch_bounds__(kSortThreads)
    k_sort_scatter(SortParams p, const uint32_t *__restrict__ offs, uint4 *__restrict__ sorted)
{
    extern __shared__ uint32_t sh_cur[];
    const uint32_t *row = offs + (size_t)blockIdx.x * p.ntiles;
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
        sh_cur[i] = row[i];
    __syncthreads();
    const int64_t b = (int64_t)blockIdx.x * p.chunk;
    const int64_t e = min(p.n, b + p.chunk);
    const float *__restrict__ pos = p.pos;
    const uint32_t mx = (1u << p.lx) - 1u, my = (1u << p.ly) - 1u, mz = (1u << p.lz) - 1u;
    for (int64_t i0 = b + threadIdx.x; i0 < e; i0 += (int64_t)kSortUnroll * blockDim.x) {
        float v[kSortUnroll][3];
        float m[kSortUnroll];
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++) {
            const int64_t i = i0 + (int64_t)u * blockDim.x;
            if (i < e) {
                v[u][0] = __ldg(pos + 3 * i);
                v[u][1] = __ldg(pos + 3 * i + 1);
                v[u][2] = __ldg(pos + 3 * i + 2);
                m[u] = VARMASS ? __ldg(p.masses + i) : 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++) {
            const int64_t i = i0 + (int64_t)u * blockDim.x;
            if (i >= e)
                break;
            int c[3];
            float d[3];
            uint32_t t;
            if (!particle_cell(p, v[u][0], v[u][1], v[u][2], c, d, t) || !isfinite(m[u]))
                continue;
            const uint32_t slot = atomicAdd(&sh_cur[t], 1u);
            uint4 w;
            w.x = (((uint32_t)c[0] & mx) << 24) | frac_to_q24(d[0]);
            w.y = (((uint32_t)c[1] & my) << 24) | frac_to_q24(d[1]);
            w.z = (((uint32_t)c[2] & mz) << 24) | frac_to_q24(d[2]);
            w.w = VARMASS ? __float_as_uint(m[u]) : 0u;
            sorted[slot] = w;
        }
    }
}

// Halo face layout of one tile (SX = TX+1 etc.; e = element index):
//   X face, local x = ext_x:        e = y*SZ + z                  y<=ext_y, z<=ext_z
//   Y face, local y = ext_y:        e = SY*SZ + x*SZ + z          x<ext_x,  z<=ext_z
//   Z face, local z = ext_z:        e = SY*SZ + TX*SZ + x*TY + y  x<ext_x,  y<ext_y
template <int TX, int TY, int TZ>
struct HaloLayout {
    static constexpr int SX = TX + 1, SY = TY + 1, SZ = TZ + 1;
    static constexpr int NX = SY * SZ;
    static constexpr int NY = TX * SZ;
    static constexpr int NZ = TX * TY;
    static constexpr int N = NX + NY + NZ;

    // Local (x, y, z) of halo element e; false where the element is unused.
    __device__ __forceinline__ static bool decode(int e, int ex, int ey, int ez, int &x, int &y,
                                                  int &z)
    {
        if (e < NX) {
            x = ex;
            y = e / SZ;
            z = e - y * SZ;
            return y <= ey && z <= ez;
        }
        e -= NX;
        if (e < NY) {
            x = e / SZ;
            z = e - x * SZ;
            y = ey;
            return x < ex && z <= ez;
        }
        e -= NY;
        x = e / TY;
        y = e - x * TY;
        z = ez;
        return x < ex && y < ey;
    }
};

struct TileParams {
    int dims;
    int64_t plane;
    int row;
    int nty, ntz;
    float mass;          // uniform mass
    double inv_cells;    // 1 / N^3
};

constexpr int kTileThreads = 512;

template <int TX, int TY, int TZ, bool VARMASS, bool CLEAN>
__global__ void __launch_bounds__(kTileThreads)
    k_tile_deposit(TileParams p, const uint4 *__restrict__ sorted,
                   const uint32_t *__restrict__ tile_start, const DeviceStatus *__restrict__ st,
                   float *__restrict__ grid, float *__restrict__ halo)
{
    using HL = HaloLayout<TX, TY, TZ>;
    constexpr int SX = HL::SX, SY = HL::SY, SZ = HL::SZ;
    constexpr int NACC = SX * SY * SZ;
    extern __shared__ float acc[];

    const int t = blockIdx.x;
    const int tz = t % p.ntz;
    const int ty = (t / p.ntz) % p.nty;
    const int tx = t / (p.ntz * p.nty);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    const int ex = min(TX, p.dims - x0), ey = min(TY, p.dims - y0), ez = min(TZ, p.dims - z0);

    for (int i = threadIdx.x; i < NACC; i += blockDim.x)
        acc[i] = 0.f;
    __syncthreads();

    const uint32_t s0 = tile_start[t], s1 = tile_start[t + 1];
    for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
        const uint4 w = sorted[i];
        const float dx = q24_to_frac(w.x), dy = q24_to_frac(w.y), dz = q24_to_frac(w.z);
        const float m = VARMASS ? __uint_as_float(w.w) : p.mass;
        const int base = ((int)(w.x >> 24) * SY + (int)(w.y >> 24)) * SZ + (int)(w.z >> 24);
        const float tx_ = 1.f - dx, ty_ = 1.f - dy, tz_ = 1.f - dz;
        // Weight order follows fieldize.cpp:77-84: ((m*wx)*wy)*wz.
        const float mtx = m * tx_, mdx = m * dx;
        const float a00 = mtx * ty_, a10 = mdx * ty_, a01 = mtx * dy, a11 = mdx * dy;
        atomicAdd(&acc[base], a00 * tz_);
        atomicAdd(&acc[base + SY * SZ], a10 * tz_);
        atomicAdd(&acc[base + SZ], a01 * tz_);
        atomicAdd(&acc[base + SY * SZ + SZ], a11 * tz_);
        atomicAdd(&acc[base + 1], a00 * dz);
        atomicAdd(&acc[base + SY * SZ + 1], a10 * dz);
        atomicAdd(&acc[base + SZ + 1], a01 * dz);
        atomicAdd(&acc[base + SY * SZ + SZ + 1], a11 * dz);
    }
    __syncthreads();

    // Interior: every real cell of the grid belongs to exactly one tile.
    const float mean = (float)(st->pass_mass * p.inv_cells);
    for (int i = threadIdx.x; i < TX * TY * TZ; i += blockDim.x) {
        const int x = i / (TY * TZ);
        const int y = (i / TZ) % TY;
        const int z = i % TZ;
        if (x < ex && y < ey && z < ez) {
            const float v = acc[(x * SY + y) * SZ + z] - mean;
            float *dst = grid + cell_index(p.plane, p.row, x0 + x, y0 + y, z0 + z);
            if (CLEAN)
                *dst = v;
            else
                *dst += v;
        }
    }
    // Halo faces to scratch (zeros where unused).
    float *h = halo + (size_t)t * HL::N;
    for (int e = threadIdx.x; e < HL::N; e += blockDim.x) {
        int x, y, z;
        const bool ok = HL::decode(e, ex, ey, ez, x, y, z);
        h[e] = ok ? acc[(x * SY + y) * SZ + z] : 0.f;
    }
}

template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(256)
    k_halo_merge(TileParams p, const float *__restrict__ halo, float *__restrict__ grid)
{
    using HL = HaloLayout<TX, TY, TZ>;
    const int t = blockIdx.x;
    const int tz = t % p.ntz;
    const int ty = (t / p.ntz) % p.nty;
    const int tx = t / (p.ntz * p.nty);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    const int ex = min(TX, p.dims - x0), ey = min(TY, p.dims - y0), ez = min(TZ, p.dims - z0);
    const float *h = halo + (size_t)t * HL::N;
    for (int e = threadIdx.x; e < HL::N; e += blockDim.x) {
        const float v = h[e];
        if (v == 0.f)
            continue;
        int x, y, z;
        if (!HL::decode(e, ex, ey, ez, x, y, z))
            continue;
        int gx = x0 + x, gy = y0 + y, gz = z0 + z;
        if (gx >= p.dims)
            gx -= p.dims;
        if (gy >= p.dims)
            gy -= p.dims;
        if (gz >= p.dims)
            gz -= p.dims;
        atomicAdd(grid + cell_index(p.plane, p.row, gx, gy, gz), v);
    }
}

int ilog2(int v)
{
    int l = 0;
    while ((1 << l) < v)
        l++;
    return l;
}

template <int TX, int TY, int TZ>
cudaError_t launch_tile_kernels(const DepositGeom &g, const DepositArgs &a,
                                DepositScratch &s, DeviceStatus *dstat, cudaStream_t stream,
                                int64_t *launches, StageHook hook, void *hook_user)
{
    TileParams tp;
    tp.dims = g.grid.dims;
    tp.plane = g.grid.plane;
    tp.row = g.grid.row;
    tp.nty = g.nty;
    tp.ntz = g.ntz;
    tp.mass = a.mass;
    const double n = (double)g.grid.dims;
    tp.inv_cells = 1.0 / (n * n * n);
    const size_t smem = sizeof(float) * (TX + 1) * (TY + 1) * (TZ + 1);
    const bool var = a.masses != nullptr;
    cudaError_t err;
#define GENPK_TILE_LAUNCH(V, C)                                                                \
    do {                                                                                       \
        auto kern = k_tile_deposit<TX, TY, TZ, V, C>;                                          \
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,          \
                                   (int)smem);                                                 \
        if (err != cudaSuccess)                                                                \
            return err;                                                                        \
        kern<<<g.ntiles, kTileThreads, smem, stream>>>(tp, s.sorted, s.tile_start, dstat,      \
                                                      a.grid, s.halo);                         \
    } while (0)
    if (var && a.clean)
        GENPK_TILE_LAUNCH(true, true);
    else if (var)
        GENPK_TILE_LAUNCH(true, false);
    else if (a.clean)
        GENPK_TILE_LAUNCH(false, true);
    else
        GENPK_TILE_LAUNCH(false, false);
#undef GENPK_TILE_LAUNCH
    (*launches)++;
    if (hook)
        hook(hook_user, "dep_tile");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    k_halo_merge<TX, TY, TZ><<<g.ntiles, 256, 0, stream>>>(tp, s.halo, a.grid);
    (*launches)++;
    if (hook)
        hook(hook_user, "dep_halo");
    return cudaGetLastError();
}

}  // namespace

bool deposit_tile_supported(int tx, int ty, int tz)
{
    return (tx == 8 && ty == 8 && tz == 8) || (tx == 16 && ty == 16 && tz == 16) ||
           (tx == 16 && ty == 32 && tz == 32) || (tx == 32 && ty == 32 && tz == 32);
}

int halo_floats(int tx, int ty, int tz)
{
    return (ty + 1) * (tz + 1) + tx * (tz + 1) + tx * ty;
}

TileShape deposit_default_tile(int dims, int64_t n)
{
    (void)n;
    if (dims <= 64)
        return {8, 8, 8};
    if (dims <= 512)
        return {16, 16, 16};
    return {32, 32, 32};
}

size_t deposit_hist_smem(const DepositGeom &g)
{
    return sizeof(uint32_t) * (size_t)g.ntiles;
}

int deposit_sort_ctas(const DepositGeom &g, int64_t n, int num_sms)
{
    const size_t smem = deposit_hist_smem(g) + 1024;
    int per_sm = (int)std::min<size_t>(4, (200 * 1024) / std::max<size_t>(smem, 1));
    per_sm = std::max(per_sm, 1);
    const int64_t want = (n + 4095) / 4096;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms * per_sm, want));
}

cudaError_t deposit_pass(const DepositGeom &g, const DepositArgs &a, DepositScratch &s,
                         DeviceStatus *dstat, int sort_ctas, cudaStream_t stream,
                         int64_t *launches, StageHook hook, void *hook_user)
{
    auto mark = [&](const char *name) {
        (*launches)++;
        if (hook)
            hook(hook_user, name);
    };
    SortParams sp;
    sp.pos = a.pos;
    sp.masses = a.masses;
    sp.n = a.n;
    sp.chunk = (a.n + sort_ctas - 1) / sort_ctas;
    if (sp.chunk < 1)
        sp.chunk = 1;
    sp.dims = g.grid.dims;
    sp.uh = g.units_hi;
    sp.ul = g.units_lo;
    sp.lx = ilog2(g.tx);
    sp.ly = ilog2(g.ty);
    sp.lz = ilog2(g.tz);
    sp.nty = g.nty;
    sp.ntz = g.ntz;
    sp.ntiles = g.ntiles;
    const size_t hsmem = deposit_hist_smem(g);
    cudaError_t err;
    if ((err = cudaFuncSetAttribute(k_sort_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)hsmem)) != cudaSuccess)
        return err;
    k_sort_hist<<<sort_ctas, kSortThreads, hsmem, stream>>>(sp, s.hist, s.mass_part, dstat);
    mark("dep_hist");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    const int tb = 256, tgrid = (g.ntiles + tb - 1) / tb;
    k_sort_colsum<<<tgrid, tb, 0, stream>>>(s.hist, sort_ctas, g.ntiles, s.totals);
    mark("dep_colsum");
    k_sort_scan<<<1, kScanThreads, 0, stream>>>(s.totals, g.ntiles, s.tile_start, s.mass_part,
                                                sort_ctas,
                                                a.masses ? -1.0 : (double)a.mass, a.field_mass,
                                                dstat);
    mark("dep_scan");
    k_sort_offsets<<<tgrid, tb, 0, stream>>>(s.hist, sort_ctas, g.ntiles, s.tile_start);
    mark("dep_offsets");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    if (a.masses) {
        if ((err = cudaFuncSetAttribute(k_sort_scatter<true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)hsmem)) != cudaSuccess)
            return err;
        k_sort_scatter<true><<<sort_ctas, kSortThreads, hsmem, stream>>>(sp, s.hist, s.sorted);
    } else {
        if ((err = cudaFuncSetAttribute(k_sort_scatter<false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)hsmem)) != cudaSuccess)
            return err;
        k_sort_scatter<false><<<sort_ctas, kSortThreads, hsmem, stream>>>(sp, s.hist, s.sorted);
    }
    mark("dep_scatter");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    if (g.tx == 8)
        return launch_tile_kernels<8, 8, 8>(g, a, s, dstat, stream, launches, hook,
                                                hook_user);
    if (g.tx == 16 && g.ty == 16)
        return launch_tile_kernels<16, 16, 16>(g, a, s, dstat, stream, launches, hook,
                                                hook_user);
    if (g.tx == 16)
        return launch_tile_kernels<16, 32, 32>(g, a, s, dstat, stream, launches, hook,
                                                hook_user);
    return launch_tile_kernels<32, 32, 32>(g, a, s, dstat, stream, launches, hook,
                                                hook_user);
}

}  // namespace genpk
