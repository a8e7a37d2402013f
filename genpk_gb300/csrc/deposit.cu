// deposit.cu -- CIC mass assignment (the GPU counterpart of fieldize.cpp:46-113).
//
// A deposit pass over n particles is a counting sort into cell tiles followed
// by one CTA per tile accumulating in shared memory:
//
//   k_sort_hist       each CTA owns a contiguous particle range; it computes
//                     every particle's cell (two-product split, split_q28),
//                     counts particles per tile in a shared histogram and
//                     writes the histogram row to scratch; it also sums the
//                     masses (Kahan, FP32 -> FP64) and takes their maximum.
//   k_sort_colsum     per tile: total over the CTA rows.
//   k_sort_scan       one CTA: exclusive scan of the tile totals -> tile_start;
//                     the pass mass, the fixed-point scale 2^s and the pass
//                     mean in fixed point.
//   k_sort_offsets    per tile: histogram rows -> each CTA's first slot.
//   k_sort_scatter    re-reads the range and writes every particle, packed as
//                     tile-local cell + 28-bit fraction per axis (+ mass bits),
//                     to its slot.
//   (grids with more tiles than a shared histogram holds run both kernels with
//    global counters instead.)
//   k_tile_deposit    one CTA per tile: each particle adds its eight CIC
//                     weights, rounded to integers of 2^-s mass units, to a
//                     (T+1)^3 block of 64-bit shared accumulators.  Integer
//                     sums are exact and independent of order, so the deposit
//                     is bit-reproducible.  Cells strictly inside the tile are
//                     final: (sum - mean) is converted to FP32 once and stored.
//                     The tile's low faces and its +1 halo layer go to scratch
//                     as 64-bit sums.
//   k_face_gather     per tile: every low-face cell adds the halo sums the
//                     (up to 7) lower neighbours hold for it, in a fixed order,
//                     and stores (sum - mean) as FP32.
//
// A grouped pass runs the same kernels once for several boxes of one grid size
// (a batch of uneven boxes): the sort CTAs are shared out over the boxes'
// particles, the per-tile kernels take the box from blockIdx.y, the scan and
// the finish one CTA or thread per box.  Record slots are global across the
// boxes (box b's tile starts are offset by its first record).
//
// No global float atomics are involved and no grid memset is needed: every real
// cell is written exactly once per pass.  Subtracting the pass mean (in fixed
// point, before the single rounding) keeps the FP32 r2c accurate; it changes
// only the excluded k = 0 mode.  The mean is rounded to 24 significant bits so
// that an empty cell holds exactly -mean in FP32 and reads back as exactly 0.
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

namespace genpk {

cudaError_t ensure_dynamic_smem(const void *func, size_t bytes)
{
    // the limit is kept per device (a process may drive several GPUs)
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess)
        return err;
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> limit;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limit[std::make_pair(dev, func)];
    if (bytes <= cur)
        return cudaSuccess;
    err = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err == cudaSuccess)
        cur = bytes;
    return err;
}

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
    float umass;     // uniform mass when masses == nullptr
    int corner;      // accumulate the exact (N/2,N/2,N/2) mode (even grids)
};

// Where a sort CTA's particles come from: the one box of a pass, or the boxes
// of a grouped pass (CTAs [cta0[b], cta0[b+1]) read box b; an empty box has
// none).  Both are passed by value in the kernel parameters.
struct OneBox {
    SortParams p;
    __device__ __forceinline__ int box_of(int) const { return 0; }
    __device__ __forceinline__ SortParams params(int) const { return p; }
    __device__ __forceinline__ int first_cta(int) const { return 0; }
};

struct BoxGroup {
    int nbox;
    int cta0[kMaxGroupBoxes + 1];
    SortParams p[kMaxGroupBoxes];
    __device__ __forceinline__ int box_of(int blk) const
    {
        int b = 0;
        while (b + 1 < nbox && blk >= cta0[b + 1])
            b++;
        return b;
    }
    __device__ __forceinline__ SortParams params(int b) const { return p[b]; }
    __device__ __forceinline__ int first_cta(int b) const { return cta0[b]; }
};

// Sort-CTA rows of each box in the histogram (k_sort_colsum, k_sort_offsets:
// box = blockIdx.y), and what the scan needs per box (box = blockIdx.x):
// its rows, mass kind, uniform mass and first record.
struct BoxRows {
    int first[kMaxGroupBoxes + 1];
};

struct ScanBoxes {
    int first[kMaxGroupBoxes + 1];
    int var[kMaxGroupBoxes];  // the particles carry masses
    double umass[kMaxGroupBoxes];
    long long rec0[kMaxGroupBoxes];
};

// Threads of a sort CTA (a CTA's particle range does not depend on them).
// 1024 per CTA: at one CTA per SM (the long per-tile runs that let the
// scatter's 16-byte records share L2 sectors) 32 warps cover the loads'
// latency.  Against 512, timed in one run: the histogram pass 0.20 -> 0.14 ms
// for 27 M random particles on 256^3, the scatter 1.17 -> 1.00 ms on the 512^3
// lattice, the 16-box batch 6.1 -> 5.4 ms.
constexpr int kSortThreads = 1024;
constexpr int kSortUnroll = 4;
constexpr uint32_t kNoTile = 0xffffffffu;

// Cell, 28-bit fraction and tile of one particle (split_q28, as the window
// engine splits it); false for a particle that must be skipped.
__device__ __forceinline__ bool particle_cell(const SortParams &p, float x, float y, float z,
                                              float m, AxisQ a[3], uint32_t &tile)
{
    if (!finite3(x, y, z) || !isfinite(m))
        return false;
    const float lim = 1.0e9f;
    if (fabsf(x * p.uh) > lim || fabsf(y * p.uh) > lim || fabsf(z * p.uh) > lim)
        return false;
    a[0] = split_q28(x, p.uh, p.ul, p.dims);
    a[1] = split_q28(y, p.uh, p.ul, p.dims);
    a[2] = split_q28(z, p.uh, p.ul, p.dims);
    tile = ((uint32_t)(a[0].cell >> p.lx) * (uint32_t)p.nty + (uint32_t)(a[1].cell >> p.ly)) *
               (uint32_t)p.ntz +
           (uint32_t)(a[2].cell >> p.lz);
    return true;
}

// Per-CTA mass sum (FP64) and max |mass| (float bits) after the particle loop.
__device__ __forceinline__ void block_mass(float msum, float mc, float mmax, double *mass_part,
                                           DeviceStatus *st)
{
    __shared__ double sh_mass[32];
    __shared__ float sh_max[32];
    double md = warp_sum_d((double)msum - (double)mc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
    if ((threadIdx.x & 31) == 0) {
        sh_mass[threadIdx.x >> 5] = md;
        sh_max[threadIdx.x >> 5] = mmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        float mx = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            s += sh_mass[w];
            mx = fmaxf(mx, sh_max[w]);
        }
        mass_part[blockIdx.x] = s;
        if (mx > 0.f)
            atomicMax(&st->max_mass_bits, __float_as_uint(mx));
    }
}

// True when some lane's tile equals the previous lane's (a run of particles in
// one tile, as spatially ordered input gives).  Without one, the lanes take
// their tile slots with one shared atomic each: __match_any_sync over 32
// distinct tiles (random order, the sorted engine's usual input) costs more
// than it merges.  Slots within a tile may then come in any order; the tile
// sums are exact integers, so the grid does not depend on it.
__device__ __forceinline__ bool warp_has_tile_runs(uint32_t t)
{
    const int lane = threadIdx.x & 31;
    const uint32_t prev = __shfl_up_sync(0xffffffffu, t, 1);
    return __any_sync(0xffffffffu, lane > 0 && t != kNoTile && t == prev);
}

// Each warp walks its CTA's range (CTA `cta` of its box) in blocks of 32*kSortUnroll consecutive
// particles (lane l takes base + l + 32u, so every load is coalesced).  The trip
// count is warp-uniform, so warp-collective intrinsics are safe in `f`.
template <typename F>
__device__ __forceinline__ void for_each_warp_batch(const SortParams &p, int cta, F &&f)
{
    const int64_t b = (int64_t)cta * p.chunk;
    const int64_t e = min(p.n, b + p.chunk);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int64_t base = b + (int64_t)warp * 32 * kSortUnroll; base < e;
         base += (int64_t)nwarps * 32 * kSortUnroll) {
        float v[kSortUnroll][3], m[kSortUnroll];
        bool in[kSortUnroll];
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++) {
            const int64_t i = base + 32 * u + lane;
            in[u] = i < e;
            if (in[u]) {
                v[u][0] = __ldg(p.pos + 3 * i);
                v[u][1] = __ldg(p.pos + 3 * i + 1);
                v[u][2] = __ldg(p.pos + 3 * i + 2);
                m[u] = p.masses ? __ldg(p.masses + i) : 0.f;
            } else {
                v[u][0] = v[u][1] = v[u][2] = m[u] = 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < kSortUnroll; u++)
            f(in[u], v[u], m[u]);
    }
}

// Tile counts of one CTA's range: a shared histogram row (GLOBAL = false) or
// straight into global totals (GLOBAL = true, for grids with many tiles).
// Lanes of a warp that fall in the same tile are merged first
// (__match_any_sync), so spatially ordered input costs one atomic per warp.
template <bool GLOBAL, class Src>
__global__ void __launch_bounds__(kSortThreads)
    k_sort_hist(const __grid_constant__ Src src, uint32_t *__restrict__ out,
                double *__restrict__ mass_part, DeviceStatus *st)
{
    extern __shared__ uint32_t sh_hist[];
    const int box = src.box_of(blockIdx.x);
    const SortParams p = src.params(box);
    const int cta = blockIdx.x - src.first_cta(box);
    st += box;
    if (!GLOBAL) {
        for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
            sh_hist[i] = 0u;
        __syncthreads();
    }
    uint32_t *counts = GLOBAL ? out + (size_t)box * p.ntiles : sh_hist;
    const int lane = threadIdx.x & 31;
    float msum = 0.f, mc = 0.f, mmax = 0.f;
    unsigned bad = 0;
    for_each_warp_batch(p, cta, [&](bool in, const float *v, float m) {
        uint32_t t = kNoTile;
        if (in) {
            AxisQ a[3];
            if (particle_cell(p, v[0], v[1], v[2], m, a, t)) {
                const float y = m - mc;  // Kahan-compensated FP32 sum of masses
                const float s = msum + y;
                mc = (s - msum) - y;
                msum = s;
                mmax = fmaxf(mmax, fabsf(m));
            } else {
                t = kNoTile;
                bad++;
            }
        }
        if (!warp_has_tile_runs(t)) {
            if (t != kNoTile)
                atomicAdd(&counts[t], 1u);
        } else {
            const unsigned peers = __match_any_sync(0xffffffffu, t);
            if (t != kNoTile && lane == __ffs(peers) - 1)
                atomicAdd(&counts[t], (uint32_t)__popc(peers));
        }
    });
    __syncthreads();
    if (!GLOBAL) {
        uint32_t *row = out + (size_t)blockIdx.x * p.ntiles;
        for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
            row[i] = sh_hist[i];
    }
    block_mass(msum, mc, mmax, mass_part, st);
    if (bad)
        atomicAdd(&st->bad_particles, (unsigned long long)bad);
}

// The histogram is [nsort][ntiles].  Its column sums and column prefix sums
// go 32 tiles (one 128-byte row segment) per CTA, with the CTA rows split
// into kColWarps contiguous blocks, one per warp: a lane's loads are
// independent and in flight together, and a grid of 16^3 tiles at 128^3
// (512 tiles) still spreads over 16 CTAs x 32 warps.  One thread per tile
// walking all rows waited out nsort dependent round trips (90 us per pass at
// 608 rows).
constexpr int kColWarps = 32;

// Sum of rows [r0, r1) of tile t's column (0 where t is out of range).
__device__ __forceinline__ uint32_t column_block_sum(const uint32_t *hist, int ntiles, int t,
                                                     int r0, int r1)
{
    uint32_t s = 0;
    if (t < ntiles) {
#pragma unroll 8
        for (int c = r0; c < r1; c++)
            s += hist[(size_t)c * ntiles + t];
    }
    return s;
}

__global__ void __launch_bounds__(32 * kColWarps)
    k_sort_colsum(const uint32_t *__restrict__ hist, const __grid_constant__ BoxRows rows,
                  int ntiles, uint32_t *__restrict__ totals)
{
    __shared__ uint32_t part[kColWarps][33];
    const int box = blockIdx.y;
    const int nsort = rows.first[box + 1] - rows.first[box];
    hist += (size_t)rows.first[box] * ntiles;
    totals += (size_t)box * ntiles;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    const int per_warp = (nsort + kColWarps - 1) / kColWarps;
    const int r0 = min(w * per_warp, nsort), r1 = min(r0 + per_warp, nsort);
    part[w][lane] = column_block_sum(hist, ntiles, t, r0, r1);
    __syncthreads();
    if (w == 0 && t < ntiles) {
        uint32_t s = 0;
        for (int k = 0; k < kColWarps; k++)
            s += part[k][lane];
        totals[t] = s;
    }
}

constexpr int kScanThreads = 1024;

// Exclusive scan of tile totals (one CTA per box) and the per-pass constants.
// A box's tile starts begin at its first record.  Unless the box's particles
// carry masses, every one weighs its uniform mass (of either sign).
__global__ void __launch_bounds__(kScanThreads)
    k_sort_scan(const uint32_t *__restrict__ totals, int ntiles, uint32_t *__restrict__ tile_start,
                uint32_t *__restrict__ cursor, const double *__restrict__ mass_part,
                const __grid_constant__ ScanBoxes boxes, double inv_cells, double *field_mass,
                double *field_sub, DeviceStatus *st)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ uint32_t carry;
    __shared__ double sh_m[kScanThreads / 32];
    const int box = blockIdx.x;
    const int nsort = boxes.first[box + 1] - boxes.first[box];
    const double uniform_mass = boxes.umass[box];
    const bool var = boxes.var[box] != 0;
    const uint32_t rec0 = (uint32_t)boxes.rec0[box];
    totals += (size_t)box * ntiles;
    tile_start += (size_t)box * (ntiles + 1);
    if (cursor)
        cursor += (size_t)box * ntiles;
    mass_part += boxes.first[box];
    field_mass += box;
    field_sub += box;
    st += box;
    if (threadIdx.x == 0)
        carry = rec0;
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
            warp_tot[lane] = w;
        }
        __syncthreads();
        const uint32_t before = (wid ? warp_tot[wid - 1] : 0u) + carry;
        if (t < ntiles) {
            tile_start[t] = before + x - v;
            if (cursor)
                cursor[t] = before + x - v;
        }
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1)
            carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        tile_start[ntiles] = carry;

    double m = 0.0;
    if (var) {
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
        m = (double)(carry - rec0) * uniform_mass;
    }
    if (threadIdx.x == 0) {
        // Scale: the largest |mass| maps into [2^27, 2^28) units of 2^-s, so one
        // CIC weight is below 2^28 (the 32-bit shared accumulators carry at most
        // once per 2^4 adds) and 64-bit cell sums hold 2^35 full-mass particles.
        const float mref = !var ? (float)fabs(uniform_mass)
                                               : __uint_as_float(st->max_mass_bits);
        st->max_mass_bits = 0u;  // read: zero again for the next pass
        int s = 0;
        if (mref > 0.f && isfinite(mref))
            s = 27 - ilogbf(mref);
        s = max(-100, min(100, s));
        const double mf = m * inv_cells * ldexp(1.0, s);
        // Round the mean to 24 significant bits: exactly representable in FP32
        // after the final 2^-s scaling.
        long long mean_fixed;
        const double amf = fabs(mf);
        if (amf >= 16777216.0) {
            const double q = ldexp(1.0, ilogb(amf) - 23);
            mean_fixed = (long long)(rint(mf / q) * q);
        } else {
            mean_fixed = llrint(mf);
        }
        st->pass_mass = m;
        st->fx_shift = s;
        st->mean_fixed = mean_fixed;
        *field_mass += m;
        *field_sub += ldexp((double)mean_fixed, -s);
    }
}

// Histogram rows -> each CTA's first slot per tile, in place: tile t's
// column becomes tile_start[t] plus the exclusive prefix sum down the column.
// Same blocking as k_sort_colsum: block sums, an exclusive scan of the 32
// block sums per tile in shared memory, then each warp rewrites its block.
__global__ void __launch_bounds__(32 * kColWarps)
    k_sort_offsets(uint32_t *__restrict__ hist, const __grid_constant__ BoxRows rows, int ntiles,
                   const uint32_t *__restrict__ tile_start)
{
    __shared__ uint32_t part[kColWarps][33];
    const int box = blockIdx.y;
    const int nsort = rows.first[box + 1] - rows.first[box];
    hist += (size_t)rows.first[box] * ntiles;
    tile_start += (size_t)box * (ntiles + 1);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    const int per_warp = (nsort + kColWarps - 1) / kColWarps;
    const int r0 = min(w * per_warp, nsort), r1 = min(r0 + per_warp, nsort);
    part[w][lane] = column_block_sum(hist, ntiles, t, r0, r1);
    __syncthreads();
    if (w == 0) {
        uint32_t run = t < ntiles ? tile_start[t] : 0u;
        for (int k = 0; k < kColWarps; k++) {
            const uint32_t v = part[k][lane];
            part[k][lane] = run;
            run += v;
        }
    }
    __syncthreads();
    if (t >= ntiles)
        return;
    uint32_t run = part[w][lane];
    for (int c = r0; c < r1; c += 8) {  // eight loads in flight, then eight stores
        uint32_t v[8];
#pragma unroll
        for (int q = 0; q < 8; q++)
            v[q] = c + q < r1 ? hist[(size_t)(c + q) * ntiles + t] : 0u;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (c + q < r1)
                hist[(size_t)(c + q) * ntiles + t] = run;
            run += v[q];
        }
    }
}

// Packed particle: per axis (tile-local cell << 28) | 28-bit fraction (tiles
// of at most 16 cells per edge), then the mass bits.
__device__ __forceinline__ uint4 pack_particle(const AxisQ a[3], float m, uint32_t mx, uint32_t my,
                                               uint32_t mz)
{
    uint4 w;
    w.x = (((uint32_t)a[0].cell & mx) << kFracBits) | a[0].q;
    w.y = (((uint32_t)a[1].cell & my) << kFracBits) | a[1].q;
    w.z = (((uint32_t)a[2].cell & mz) << kFracBits) | a[2].q;
    w.w = __float_as_uint(m);
    return w;
}

// Writes every particle of the CTA's range to its slot in tile order.  Shared
// cursors start at this CTA's offsets (GLOBAL = false) or global cursors are
// used directly (GLOBAL = true).  Lanes in the same tile take consecutive slots
// from one atomic.  Packed particle: per axis (tile-local cell << 28) | 28-bit
// fraction; w = mass bits.
//
// On even grids it also sums the corner mode k = (N/2, N/2, N/2) of the CIC
// density exactly: that DFT coefficient is sum over particles of
// m (-1)^(x+y+z) prod_a (1 - 2 d_a) with (x, y, z) the particle's cell and d_a
// its fractions.  Each term is formed from the full two-product position in
// float-pair arithmetic and summed per thread in float pairs; each warp's total
// is rounded to an integer of 2^-(s+4) mass units and summed in 64-bit integers
// (deterministic: fixed per-thread order, integer sums across warps).  The last log-k bin holds only
// this mode, so its value must not carry the FP32 grid's rounding noise.
template <bool GLOBAL, class Src>
__global__ void __launch_bounds__(kSortThreads)
    k_sort_scatter(const __grid_constant__ Src src, uint32_t *__restrict__ offs,
                   uint4 *__restrict__ sorted, DeviceStatus *st)
{
    extern __shared__ uint32_t sh_cur[];
    const int box = src.box_of(blockIdx.x);
    const SortParams p = src.params(box);
    const int cta = blockIdx.x - src.first_cta(box);
    st += box;
    if (!GLOBAL) {
        const uint32_t *row = offs + (size_t)blockIdx.x * p.ntiles;
        for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
            sh_cur[i] = row[i];
        __syncthreads();
    }
    uint32_t *cur = GLOBAL ? offs + (size_t)box * p.ntiles : sh_cur;
    const uint32_t mx = (1u << p.lx) - 1u, my = (1u << p.ly) - 1u, mz = (1u << p.lz) - 1u;
    const int lane = threadIdx.x & 31;
    // Corner terms in 2^-(s+4) mass units (|term| < 2^32), summed per thread as
    // a float pair and converted to an integer once per warp.
    const float mscale = ldexpf(1.f, st->fx_shift + 4);
    f2sum alt = {0.f, 0.f};
    for_each_warp_batch(p, cta, [&](bool in, const float *v, float m) {
        uint32_t t = kNoTile;
        AxisQ a[3];
        a[0] = a[1] = a[2] = AxisQ{0, 0u, 1.f, 0.f};
        if (in && !particle_cell(p, v[0], v[1], v[2], m, a, t))
            t = kNoTile;
        uint32_t slot = 0;
        if (!warp_has_tile_runs(t)) {
            if (t != kNoTile)
                slot = atomicAdd(&cur[t], 1u);
        } else {
            const unsigned peers = __match_any_sync(0xffffffffu, t);
            const int leader = __ffs(peers) - 1;
            uint32_t slot0 = 0;
            if (t != kNoTile && lane == leader)
                slot0 = atomicAdd(&cur[t], (uint32_t)__popc(peers));
            slot = __shfl_sync(0xffffffffu, slot0, leader) + __popc(peers & ((1u << lane) - 1u));
        }
        if (t != kNoTile) {
            // (the mass word carries a uniform mass too, for grouped passes)
            sorted[slot] = pack_particle(a, p.masses ? m : p.umass, mx, my, mz);
            if (p.corner) {
                const float mm = (p.masses ? m : p.umass) * mscale;
                f2sum u = corner_factor_q(a[0], a[1], a[2]);
                const float h = __fmul_rn(u.hi, mm);
                u = f2sum{h, fmaf(u.hi, mm, -h) + u.lo * mm};
                f2_accumulate(alt, f2_signed(u, a[0].cell ^ a[1].cell ^ a[2].cell));
            }
        }
    });
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
}

// Halo layer of one tile (the cells at local x = ext_x, y = ext_y or z = ext_z),
// stored as 64-bit sums.  S* = T* + 1.
//   X face (x = ext_x):              e = y*SZ + z                   y<=ext_y, z<=ext_z
//   Y face (y = ext_y, x < ext_x):   e = NX + x*SZ + z              z<=ext_z
//   Z face (z = ext_z, x, y inside): e = NX + NY + x*TY + y
// Low faces of one tile (local x = 0, y = 0 or z = 0), 64-bit sums:
//   A (x = 0):                       e = y*TZ + z
//   B (y = 0, x >= 1):               e = TY*TZ + x*TZ + z
//   C (z = 0, x >= 1, y >= 1):       e = TY*TZ + TX*TZ + x*TY + y
template <int TX, int TY, int TZ>
struct TileLayout {
    static constexpr int SX = TX + 1, SY = TY + 1, SZ = TZ + 1;
    static constexpr int NACC = SX * SY * SZ;
    static constexpr int NX = SY * SZ, NY = TX * SZ, NZ = TX * TY;
    static constexpr int NHALO = NX + NY + NZ;
    static constexpr int NFACE = TY * TZ + TX * TZ + TX * TY;

    __device__ __forceinline__ static int acc_index(int x, int y, int z)
    {
        return (x * SY + y) * SZ + z;
    }

    __device__ __forceinline__ static bool halo_decode(int e, int ex, int ey, int ez, int &x,
                                                       int &y, int &z)
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

    // Inverse of halo_decode for a cell on the halo layer.
    __device__ __forceinline__ static int halo_encode(int x, int y, int z, int ex, int ey)
    {
        if (x == ex)
            return y * SZ + z;
        if (y == ey)
            return NX + x * SZ + z;
        return NX + NY + x * TY + y;
    }

    __device__ __forceinline__ static bool face_decode(int e, int ex, int ey, int ez, int &x,
                                                       int &y, int &z)
    {
        if (e < TY * TZ) {
            x = 0;
            y = e / TZ;
            z = e - y * TZ;
            return y < ey && z < ez;
        }
        e -= TY * TZ;
        if (e < TX * TZ) {
            x = e / TZ;
            z = e - x * TZ;
            y = 0;
            return x >= 1 && x < ex && z < ez;
        }
        e -= TX * TZ;
        x = e / TY;
        y = e - x * TY;
        z = 0;
        return x >= 1 && x < ex && y >= 1 && y < ey;
    }
};

struct TileParams {
    int dims;
    int64_t plane;
    int row;
    int ntx, nty, ntz;
    float mass;  // uniform mass when the particles carry none
};

constexpr int kTileThreads = 512;

__device__ __forceinline__ float fixed_to_float(long long v, float inv_scale)
{
    // One rounding (int64 -> float), then an exact power-of-two scaling.
    return i64_to_f32_rn(v) * inv_scale;
}

__device__ __forceinline__ void tile_coords(const TileParams &p, int t, int &tx, int &ty, int &tz)
{
    tz = t % p.ntz;
    ty = (t / p.ntz) % p.nty;
    tx = t / (p.ntz * p.nty);
}

// 64-bit cell sum kept as two 32-bit shared words: lo takes each weight with a
// native 32-bit atomic, and the rare carry out of it (weights are < 2^28, so at
// most one add in 2^4 carries) goes to hi.  Exact and order-independent.
// A positive weight is added whatever its value (testing for zero, a particle
// on a cell face, cost more than the rare empty add: 0.218 -> 0.213 ms for
// 27 M particles on 256^3); a negative one skips zero, since its high-word
// term assumes w > 0.
__device__ __forceinline__ void acc_add(unsigned *lo, unsigned *hi, int idx, unsigned w, bool neg)
{
    if (neg && w == 0u)
        return;
    if (!neg) {
        const unsigned old = atomicAdd(&lo[idx], w);
        if (old + w < old)
            atomicAdd(&hi[idx], 1u);
    } else {  // adding -w: lo += 2^32 - w, hi += carry - 1
        const unsigned wl = 0u - w;
        const unsigned old = atomicAdd(&lo[idx], wl);
        if (!(old + wl < old))
            atomicAdd(&hi[idx], 0xffffffffu);
    }
}

__device__ __forceinline__ long long acc_get(const unsigned *lo, const unsigned *hi, int idx)
{
    return (long long)(((unsigned long long)hi[idx] << 32) | lo[idx]);
}

// Tile blockIdx.x of box blockIdx.y (grid_stride floats between the boxes' grids).
template <int TX, int TY, int TZ, bool VARMASS, bool CLEAN>
__global__ void __launch_bounds__(kTileThreads)
    k_tile_deposit(TileParams p, const uint4 *__restrict__ sorted,
                   const uint32_t *__restrict__ tile_start, DeviceStatus *__restrict__ st,
                   float *__restrict__ grid, long long *__restrict__ faces,
                   long long *__restrict__ halo, int64_t grid_stride)
{
    using L = TileLayout<TX, TY, TZ>;
    extern __shared__ unsigned acc_words[];
    unsigned *lo = acc_words, *hi = acc_words + L::NACC;
    const int t = blockIdx.x;
    {
        const int box = blockIdx.y;
        const int ntiles = p.ntx * p.nty * p.ntz;
        tile_start += (size_t)box * (ntiles + 1);
        st += box;
        grid += (size_t)box * (size_t)grid_stride;
        faces += (size_t)box * ntiles * L::NFACE;
        halo += (size_t)box * ntiles * L::NHALO;
    }
    int tx, ty, tz;
    tile_coords(p, t, tx, ty, tz);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    const int ex = min(TX, p.dims - x0), ey = min(TY, p.dims - y0), ez = min(TZ, p.dims - z0);
    for (int i = threadIdx.x; i < 2 * L::NACC; i += blockDim.x)
        acc_words[i] = 0u;
    __syncthreads();

    const int s = st->fx_shift;
    const float inv_scale = ldexpf(1.f, -s);
    // Weights in 2^-s mass units with s = 154 - emax (common.cuh pair_w / z_mass /
    // corner_w, as the window engine computes them).
    const int emax = 154 - s;
    const unsigned ubits = __float_as_uint(p.mass);
    const unsigned umant = (ubits & 0x7fffffu) | 0x800000u;
    const int uef = (int)((ubits >> 23) & 0xffu);
    const bool uneg = (ubits >> 31) != 0u;
    const uint32_t s0 = tile_start[t], s1 = tile_start[t + 1];
    for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
        const uint4 w = sorted[i];
        unsigned mant = umant;
        int ef = uef;
        bool neg = uneg;
        if (VARMASS) {
            const unsigned mb = w.w;
            ef = (int)((mb >> 23) & 0xffu);
            mant = (mb & 0x7fffffu) | 0x800000u;
            neg = (mb >> 31) != 0u;
        }
        if (ef == 0)  // zero or subnormal mass deposits nothing
            continue;
        const int dsh = max(emax - ef, 0);
        const uint32_t qx = w.x & (kFracOne - 1u), qy = w.y & (kFracOne - 1u),
                       qz = w.z & (kFracOne - 1u);
        const uint32_t rx = kFracOne - qx, ry = kFracOne - qy, rz = kFracOne - qz;
        const int base = L::acc_index((int)(w.x >> kFracBits), (int)(w.y >> kFracBits),
                                      (int)(w.z >> kFracBits));
        constexpr int DX = L::SY * L::SZ, DY = L::SZ;
        const uint32_t p00 = pair_w(rx, ry), p10 = pair_w(qx, ry), p01 = pair_w(rx, qy),
                       p11 = pair_w(qx, qy);
        const uint32_t z0 = z_mass(rz, mant, dsh), z1 = z_mass(qz, mant, dsh);
        acc_add(lo, hi, base, corner_w(p00, z0), neg);
        acc_add(lo, hi, base + DX, corner_w(p10, z0), neg);
        acc_add(lo, hi, base + DY, corner_w(p01, z0), neg);
        acc_add(lo, hi, base + DX + DY, corner_w(p11, z0), neg);
        acc_add(lo, hi, base + 1, corner_w(p00, z1), neg);
        acc_add(lo, hi, base + DX + 1, corner_w(p10, z1), neg);
        acc_add(lo, hi, base + DY + 1, corner_w(p01, z1), neg);
        acc_add(lo, hi, base + DX + DY + 1, corner_w(p11, z1), neg);
    }
    __syncthreads();

    // Cells strictly inside the tile (no low face): final value.
    const long long mean = st->mean_fixed;
    for (int i = threadIdx.x; i < TX * TY * TZ; i += blockDim.x) {
        const int x = i / (TY * TZ);
        const int y = (i / TZ) % TY;
        const int z = i % TZ;
        if (x >= 1 && y >= 1 && z >= 1 && x < ex && y < ey && z < ez) {
            const long long sum = acc_get(lo, hi, L::acc_index(x, y, z));
            const float v = fixed_to_float(sum - mean, inv_scale);
            float *dst = grid + cell_index(p.plane, p.row, x0 + x, y0 + y, z0 + z);
            if (CLEAN)
                *dst = v;
            else
                *dst += v;
        }
    }
    long long *f = faces + (size_t)t * L::NFACE;
    for (int e = threadIdx.x; e < L::NFACE; e += blockDim.x) {
        int x, y, z;
        if (L::face_decode(e, ex, ey, ez, x, y, z))
            f[e] = acc_get(lo, hi, L::acc_index(x, y, z));
    }
    long long *h = halo + (size_t)t * L::NHALO;
    for (int e = threadIdx.x; e < L::NHALO; e += blockDim.x) {
        int x, y, z;
        if (L::halo_decode(e, ex, ey, ez, x, y, z))
            h[e] = acc_get(lo, hi, L::acc_index(x, y, z));
    }
}

// Extent of tile index ti along an axis of `dims` cells with tiles of T.
__device__ __forceinline__ int tile_ext(int ti, int T, int dims)
{
    return min(T, dims - ti * T);
}

template <int TX, int TY, int TZ, bool CLEAN>
__global__ void __launch_bounds__(256)
    k_face_gather(TileParams p, const long long *__restrict__ faces,
                  const long long *__restrict__ halo, DeviceStatus *__restrict__ st,
                  float *__restrict__ grid, int64_t grid_stride)
{
    using L = TileLayout<TX, TY, TZ>;
    const int t = blockIdx.x;
    {
        const int box = blockIdx.y;
        const int ntiles = p.ntx * p.nty * p.ntz;
        st += box;
        grid += (size_t)box * (size_t)grid_stride;
        faces += (size_t)box * ntiles * L::NFACE;
        halo += (size_t)box * ntiles * L::NHALO;
    }
    int tx, ty, tz;
    tile_coords(p, t, tx, ty, tz);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    const int ex = min(TX, p.dims - x0), ey = min(TY, p.dims - y0), ez = min(TZ, p.dims - z0);
    // Lower neighbour along each axis (periodic) and its extent.
    const int txm = tx ? tx - 1 : p.ntx - 1;
    const int tym = ty ? ty - 1 : p.nty - 1;
    const int tzm = tz ? tz - 1 : p.ntz - 1;
    const int exm = tile_ext(txm, TX, p.dims), eym = tile_ext(tym, TY, p.dims),
              ezm = tile_ext(tzm, TZ, p.dims);
    const float inv_scale = ldexpf(1.f, -st->fx_shift);
    const long long mean = st->mean_fixed;
    const long long *f = faces + (size_t)t * L::NFACE;
    for (int e = threadIdx.x; e < L::NFACE; e += blockDim.x) {
        int a, b, c;
        if (!L::face_decode(e, ex, ey, ez, a, b, c))
            continue;
        long long sum = f[e];
        const int zmask = (a == 0 ? 1 : 0) | (b == 0 ? 2 : 0) | (c == 0 ? 4 : 0);
        // Every non-empty subset of the axes on which the cell sits on the low
        // face names one lower neighbour whose halo layer holds a share of it.
#pragma unroll
        for (int mask = 1; mask < 8; mask++) {
            if (mask & ~zmask)
                continue;
            const int sx = (mask & 1) ? txm : tx, sy = (mask & 2) ? tym : ty,
                      sz = (mask & 4) ? tzm : tz;
            const int sex = (mask & 1) ? exm : ex, sey = (mask & 2) ? eym : ey;
            const int xs = (mask & 1) ? exm : a, ys = (mask & 2) ? eym : b,
                      zs = (mask & 4) ? ezm : c;
            const int src = (sx * p.nty + sy) * p.ntz + sz;
            sum += halo[(size_t)src * L::NHALO + L::halo_encode(xs, ys, zs, sex, sey)];
        }
        const float v = fixed_to_float(sum - mean, inv_scale);
        float *dst = grid + cell_index(p.plane, p.row, x0 + a, y0 + b, z0 + c);
        if (CLEAN)
            *dst = v;
        else
            *dst += v;
    }
}

// The corner mode k = (N/2, N/2, N/2) of an even grid is sum (-1)^(x+y+z) rho(x):
// this pass's exact share, in mass units, joins the grid's running value.  (The
// subtracted mean contributes nothing: the signs balance on an even grid.)  The
// sum is zeroed for the next pass here, so no pass has to clear it first.
// One thread per box; a grouped pass also hands each box's count of skipped
// particles to bad_out and zeroes it.
__global__ void k_pass_finish(DeviceStatus *__restrict__ st, double *field_corner, int nbox,
                              unsigned long long *bad_out)
{
    const int b = threadIdx.x;
    if (b >= nbox)
        return;
    field_corner[b] += ldexp((double)st[b].alt_sum, -(st[b].fx_shift + 4));
    st[b].alt_sum = 0;
    if (bad_out) {
        bad_out[b] = st[b].bad_particles;
        st[b].bad_particles = 0;
    }
}

int ilog2(int v)
{
    int l = 0;
    while ((1 << l) < v)
        l++;
    return l;
}

// What the tile kernels of a pass write: nbox grids from `grid` on, with
// their corner sums and (grouped passes) skipped-particle counts.
struct TileTarget {
    float *grid;
    int64_t grid_stride;
    int nbox;
    float mass;  // uniform mass when !var
    bool var;    // records carry the masses
    bool clean;
    double *field_corner;
    unsigned long long *bad_out;
};

template <int TX, int TY, int TZ>
cudaError_t launch_tile_kernels(const DepositGeom &g, const TileTarget &a, DepositScratch &s,
                                DeviceStatus *dstat, cudaStream_t stream, int64_t *launches,
                                StageHook hook, void *hook_user)
{
    using L = TileLayout<TX, TY, TZ>;
    TileParams tp;
    tp.dims = g.grid.dims;
    tp.plane = g.grid.plane;
    tp.row = g.grid.row;
    tp.ntx = g.ntx;
    tp.nty = g.nty;
    tp.ntz = g.ntz;
    tp.mass = a.mass;
    const size_t smem = 2 * sizeof(unsigned) * L::NACC;
    const bool var = a.var;
    const dim3 tiles((unsigned)g.ntiles, (unsigned)a.nbox);
    cudaError_t err;
#define GENPK_TILE_LAUNCH(V, C)                                                                \
    do {                                                                                       \
        auto kern = k_tile_deposit<TX, TY, TZ, V, C>;                                          \
        err = ensure_dynamic_smem(kern, smem);                                                 \
        if (err != cudaSuccess)                                                                \
            return err;                                                                        \
        kern<<<tiles, kTileThreads, smem, stream>>>(tp, s.sorted, s.tile_start, dstat, a.grid, \
                                                   s.faces, s.halo, a.grid_stride);            \
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
    if (a.clean)
        k_face_gather<TX, TY, TZ, true><<<tiles, 256, 0, stream>>>(tp, s.faces, s.halo, dstat,
                                                                   a.grid, a.grid_stride);
    else
        k_face_gather<TX, TY, TZ, false><<<tiles, 256, 0, stream>>>(tp, s.faces, s.halo, dstat,
                                                                    a.grid, a.grid_stride);
    (*launches)++;
    if (hook)
        hook(hook_user, "dep_faces");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    k_pass_finish<<<1, ((a.nbox + 31) / 32) * 32, 0, stream>>>(dstat, a.field_corner, a.nbox,
                                                               a.bad_out);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_tile_pass(const DepositGeom &g, const TileTarget &t, DepositScratch &s,
                             DeviceStatus *dstat, cudaStream_t stream, int64_t *launches,
                             StageHook hook, void *hook_user)
{
    if (g.tx == 8)
        return launch_tile_kernels<8, 8, 8>(g, t, s, dstat, stream, launches, hook, hook_user);
    if (g.tz == 8)
        return launch_tile_kernels<16, 16, 8>(g, t, s, dstat, stream, launches, hook, hook_user);
    return launch_tile_kernels<16, 16, 16>(g, t, s, dstat, stream, launches, hook, hook_user);
}

SortParams sort_params(const DepositGeom &g, const float *pos, const float *masses, float mass,
                       int64_t n, float uh, float ul, int ctas)
{
    SortParams sp;
    sp.pos = pos;
    sp.masses = masses;
    sp.n = n;
    sp.chunk = ctas > 0 ? (n + ctas - 1) / ctas : 1;
    if (sp.chunk < 1)
        sp.chunk = 1;
    sp.dims = g.grid.dims;
    sp.uh = uh;
    sp.ul = ul;
    sp.lx = ilog2(g.tx);
    sp.ly = ilog2(g.ty);
    sp.lz = ilog2(g.tz);
    sp.nty = g.nty;
    sp.ntz = g.ntz;
    sp.ntiles = g.ntiles;
    sp.umass = mass;
    sp.corner = (g.grid.dims % 2 == 0) ? 1 : 0;
    return sp;
}

}  // namespace

// Tile edges of at most 16 cells: the packed record keeps 4 bits of tile-local
// cell beside each 28-bit fraction.
bool deposit_tile_supported(int tx, int ty, int tz)
{
    return (tx == 8 && ty == 8 && tz == 8) || (tx == 16 && ty == 16 && tz == 8) ||
           (tx == 16 && ty == 16 && tz == 16);
}

TileShape deposit_default_tile(int dims, int64_t n)
{
    (void)n;
    if (dims <= 64)
        return {8, 8, 8};
    return {16, 16, 16};
}

void deposit_scratch_sizes(const DepositGeom &g, size_t *face_elems, size_t *halo_elems)
{
    const int tx = g.tx, ty = g.ty, tz = g.tz;
    *face_elems = (size_t)g.ntiles * (size_t)(ty * tz + tx * tz + tx * ty);
    *halo_elems = (size_t)g.ntiles * (size_t)((ty + 1) * (tz + 1) + tx * (tz + 1) + tx * ty);
}

size_t deposit_hist_smem(const DepositGeom &g)
{
    return sizeof(uint32_t) * (size_t)g.ntiles;
}

bool deposit_shared_hist(const DepositGeom &g)
{
    return deposit_hist_smem(g) <= 160 * 1024;
}

int deposit_sort_ctas(const DepositGeom &g, int64_t n, int num_sms, int max_per_sm)
{
    int per_sm = std::max(1, max_per_sm);
    if (deposit_shared_hist(g)) {
        const size_t smem = deposit_hist_smem(g) + 1024;
        per_sm = (int)std::min<size_t>((size_t)per_sm, (200 * 1024) / std::max<size_t>(smem, 1));
        per_sm = std::max(per_sm, 1);
    }
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
    const OneBox src{sort_params(g, a.pos, a.masses, a.mass, a.n, g.units_hi, g.units_lo,
                                 sort_ctas)};
    BoxRows rows = {};
    rows.first[1] = sort_ctas;
    ScanBoxes sb = {};
    sb.first[1] = sort_ctas;
    sb.var[0] = a.masses ? 1 : 0;
    sb.umass[0] = (double)a.mass;
    const bool shared_hist = deposit_shared_hist(g);
    const double n3 = (double)g.grid.dims * g.grid.dims * g.grid.dims;
    cudaError_t err;
    // (max_mass_bits and alt_sum are zero here: the pass that used them last
    // zeroed them, in k_sort_scan / k_window_prep and the finishing kernels)
    const int cgrid = (g.ntiles + 31) / 32;
    const size_t hsmem = deposit_hist_smem(g);
    if (shared_hist) {
        if ((err = ensure_dynamic_smem(k_sort_hist<false, OneBox>, hsmem)) != cudaSuccess)
            return err;
        k_sort_hist<false><<<sort_ctas, kSortThreads, hsmem, stream>>>(src, s.hist, s.mass_part,
                                                                       dstat);
        mark("dep_hist");
        k_sort_colsum<<<cgrid, 32 * kColWarps, 0, stream>>>(s.hist, rows, g.ntiles, s.totals);
        mark("dep_colsum");
    } else {
        if ((err = cudaMemsetAsync(s.totals, 0, sizeof(uint32_t) * g.ntiles, stream)) !=
            cudaSuccess)
            return err;
        k_sort_hist<true><<<sort_ctas, kSortThreads, 0, stream>>>(src, s.totals, s.mass_part,
                                                                  dstat);
        mark("dep_hist");
    }
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    k_sort_scan<<<1, kScanThreads, 0, stream>>>(s.totals, g.ntiles, s.tile_start,
                                                shared_hist ? nullptr : s.cursor, s.mass_part, sb,
                                                1.0 / n3, a.field_mass, a.field_sub, dstat);
    mark("dep_scan");
    if (shared_hist) {
        k_sort_offsets<<<cgrid, 32 * kColWarps, 0, stream>>>(s.hist, rows, g.ntiles,
                                                             s.tile_start);
        mark("dep_offsets");
        if ((err = ensure_dynamic_smem(k_sort_scatter<false, OneBox>, hsmem)) != cudaSuccess)
            return err;
        k_sort_scatter<false><<<sort_ctas, kSortThreads, hsmem, stream>>>(src, s.hist, s.sorted,
                                                                         dstat);
    } else {
        k_sort_scatter<true><<<sort_ctas, kSortThreads, 0, stream>>>(src, s.cursor, s.sorted,
                                                                       dstat);
    }
    mark("dep_scatter");
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    const TileTarget t{a.grid, 0, 1, a.mass, a.masses != nullptr, a.clean, a.field_corner,
                       nullptr};
    return launch_tile_pass(g, t, s, dstat, stream, launches, hook, hook_user);
}

GroupLayout deposit_group_layout(int nbox, const GroupBox *boxes, int sort_ctas)
{
    GroupLayout lay = {};
    lay.nbox = nbox;
    int64_t total = 0;
    for (int b = 0; b < nbox; b++)
        total += boxes[b].n;
    int c = 0;
    int64_t r = 0;
    for (int b = 0; b < nbox; b++) {
        const int64_t n = boxes[b].n;
        int k = 0;
        if (n > 0) {
            const double share = (double)sort_ctas * (double)n / (double)total;
            k = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::llround(share),
                                                            (n + 4095) / 4096));
        }
        lay.cta0[b] = c;
        lay.rec0[b] = r;
        c += k;
        r += n;
    }
    lay.cta0[nbox] = c;
    lay.rec0[nbox] = r;
    return lay;
}

cudaError_t deposit_group_pass(const DepositGeom &g, const GroupLayout &lay, const GroupBox *boxes,
                               float *grid0, int64_t grid_stride, double *field_mass0,
                               double *field_sub0, double *field_corner0, DepositScratch &s,
                               DeviceStatus *st0, unsigned long long *bad_out, cudaStream_t stream,
                               int64_t *launches)
{
    const int nbox = lay.nbox;
    if (nbox < 1 || nbox > kMaxGroupBoxes || !deposit_shared_hist(g) ||
        lay.rec0[nbox] > (int64_t)0xfffffffeLL)
        return cudaErrorInvalidValue;
    BoxGroup src = {};
    BoxRows rows = {};
    ScanBoxes sb = {};
    src.nbox = nbox;
    for (int b = 0; b <= nbox; b++) {
        src.cta0[b] = lay.cta0[b];
        rows.first[b] = lay.cta0[b];
        sb.first[b] = lay.cta0[b];
    }
    for (int b = 0; b < nbox; b++) {
        const GroupBox &x = boxes[b];
        src.p[b] = sort_params(g, x.pos, x.masses, x.mass, x.n, x.units_hi, x.units_lo,
                               lay.cta0[b + 1] - lay.cta0[b]);
        sb.var[b] = x.masses ? 1 : 0;
        sb.umass[b] = (double)x.mass;
        sb.rec0[b] = (long long)lay.rec0[b];
    }
    const int ctas = lay.cta0[nbox];
    const double n3 = (double)g.grid.dims * g.grid.dims * g.grid.dims;
    const int cgrid = (g.ntiles + 31) / 32;
    const size_t hsmem = deposit_hist_smem(g);
    cudaError_t err;
    if (ctas > 0) {
        if ((err = ensure_dynamic_smem(k_sort_hist<false, BoxGroup>, hsmem)) != cudaSuccess)
            return err;
        k_sort_hist<false><<<ctas, kSortThreads, hsmem, stream>>>(src, s.hist, s.mass_part, st0);
        (*launches)++;
    }
    k_sort_colsum<<<dim3(cgrid, nbox), 32 * kColWarps, 0, stream>>>(s.hist, rows, g.ntiles,
                                                                     s.totals);
    k_sort_scan<<<nbox, kScanThreads, 0, stream>>>(s.totals, g.ntiles, s.tile_start, nullptr,
                                                   s.mass_part, sb, 1.0 / n3, field_mass0,
                                                   field_sub0, st0);
    k_sort_offsets<<<dim3(cgrid, nbox), 32 * kColWarps, 0, stream>>>(s.hist, rows, g.ntiles,
                                                                      s.tile_start);
    *launches += 3;
    if (ctas > 0) {
        if ((err = ensure_dynamic_smem(k_sort_scatter<false, BoxGroup>, hsmem)) != cudaSuccess)
            return err;
        k_sort_scatter<false><<<ctas, kSortThreads, hsmem, stream>>>(src, s.hist, s.sorted, st0);
        (*launches)++;
    }
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    // every box's records carry its mass bits, so the tile kernels read them
    const TileTarget t{grid0, grid_stride, nbox, 0.f, true, true, field_corner0, bad_out};
    return launch_tile_pass(g, t, s, st0, stream, launches, nullptr, nullptr);
}

}  // namespace genpk
