// xfft.cu -- the forward 3-D r2c FFT for N = 64..512 (powers of two) as three
// passes of our own (the GPU counterpart of the FFTW plan of
// gen-pk.cpp:186-193,233), the last one fused with the auto-spectrum binning of
// powerspectrum.c:35-111, and the adjoint's first inverse pass.
//
//   k_zfft    the r2c along z of one freshly deposited field, read straight
//             from the deposit's 64-bit accumulator (one warp per row);
//   k_yfft    the complex pass along y (cp.async tiles, Stockham stages);
//   k_xfft    the complex pass along x for every (j, kz) column, in place (the
//             layout cuFFT's 3-D R2C produces).  It runs after k_zfft + k_yfft
//             or after a batched 2-D cuFFT R2C over the x-planes (fields that
//             were converted first).  Modes: plain; binning |F|^2 of the auto
//             spectrum in the same pass, so the spectrum is read from HBM once
//             instead of twice, and clearing the used accumulator with spare
//             bandwidth; or the adjoint's inverse pass with the mode gradient
//             applied as the first stage reads each mode.
//
// k_xfft:
//
//   tiles     TZ = 4096/N consecutive columns f = j*(N/2+1) + kz (a 32 KB
//             tile of N rows x TZ complex), moved by TMA (cp.async.bulk.tensor
//             2-D loads and stores) into / out of shared memory; persistent
//             CTAs (two per SM), double-buffered loads.
//   FFT       Stockham autosort, radix 8 (one radix-2 or -4 stage last),
//             in place in the tile with a barrier between the read and write
//             half of every stage; 512 threads, each one radix-8 butterfly
//             (or two radix-4, four radix-2) per stage; twiddles from an FP32
//             table of exp(-2 pi i m/N) rounded from FP64 on the host.
//   binning   the last stage also writes v = c * p^4 * |F|^2 (p = (iw_x iw_y)
//             iw_z as in the binning kernel) into a [column][row] buffer;
//             every thread then walks 8 modes along the columns of a row
//             (|k|^2 grows with kz) with a running bin, flushing into a
//             per-warp FP32 histogram;
//             the lanes' open sums are combined by a segmented warp scan (rows
//             of a warp lie in one half of the axis, so their bins are
//             monotone); every 8 tiles the warps' histograms are summed in a
//             fixed order into the CTA's FP64 histogram; k_bin_finalize reduces
//             the CTA partials.
#include "common.cuh"
#include "internal.h"

#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <mutex>

namespace genpk {
namespace {

constexpr int kXThreads = 512;
constexpr int kXCtasPerSm = 2;
constexpr int kXTileBytes = 32 * 1024;  // N rows x (4096/N) complex
constexpr int kXMaxBins = 256;

struct XParams {
    uint4 *zero;           // region to clear (16-byte units), or null
    int64_t zero_units;
    int64_t zero_per_tile; // units cleared per tile
    int dims, hc, tz;
    int log2n;
    int n8;                // radix-8 stages before the last stage
    int ncols;             // dims * hc columns per field
    int tiles_per_field;
    int ntiles;            // tiles_per_field * nbatch
    int box_rows;          // rows per TMA box
    const float2 *tw;      // [dims] exp(-2 pi i m / dims)
    // binning (nrbins == 0: none) of the batch's single field (bin_fields = 1)
    // or of each field of the batch (bin_fields = nbatch)
    int nrbins;
    int bin_fields;
    float bpu_half;
    const uint32_t *thr;   // [nrbins + 1]
    const float *iw;       // [dims]
    const double *corner;  // exact (N/2,N/2,N/2) value per binned field, or null
    double *partial;       // [gridDim.x][bin_fields][nrbins]
    const float *gcoef;    // adjoint: [nrbins] per-bin coefficients G_b
};

// What k_xfft does around its transform: the forward pass alone, the forward
// pass binning its field's auto spectrum, or the adjoint's inverse pass, which
// first scales every mode by the P(k) loss gradient (the mode gradient
// H = G_b V_m c_m/mult_m F_m) and runs the inverse transform as
// conj(FFT(conj(H))).
constexpr int kXPlain = 0, kXBin = 1, kXGrad = 2;

// This tile's share of a region cleared alongside the x pass: units
// [t * per, (t + 1) * per) of the region's n 16-byte units, as streaming
// stores (nothing waits on them; they use HBM bandwidth that the pass's
// shared-memory-bound stages leave idle).
template <int THREADS>
__device__ __forceinline__ void zero_share(uint4 *z, int64_t n, int64_t per, int64_t t, int tid)
{
    if (z == nullptr)
        return;
    const int64_t a = t * per;
    const int64_t e = min(a + per, n);
    for (int64_t u = a + tid; u < e; u += THREADS)
        __stcs(z + u, make_uint4(0u, 0u, 0u, 0u));
}

struct ColInfo {
    int r2;      // ky^2 + kz^2, or -1 for a column past the end
    float iwj;   // iw(ky)
    float iwz;   // iw(kz)
    float w;     // mode weight: 1 on the kz = 0 and kz = N/2 planes, else 2
    int special; // 1: (j, kz) = (0, 0) (row 0 is the skipped k = 0 mode);
                 // 2: (j, kz) = (N/2, N/2) (row N/2 is the exact corner mode)
    int run;     // 1: kz = 0, a new run of consecutive kz begins (new ky)
    int pad[2];
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

// Bounded wait (~2^31 clocks, about a second): false if it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > (1ll << 31))
            return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y, const void *src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::
                     "l"(map),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit()
{
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void bulk_wait_read_all()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    return make_float2(a.x + b.x, a.y + b.y);
}

__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    return make_float2(a.x - b.x, a.y - b.y);
}

// multiply by -i
__device__ __forceinline__ float2 mul_mi(float2 a)
{
    return make_float2(a.y, -a.x);
}

// Forward R-point DFTs in registers, natural order in and out.
__device__ __forceinline__ void dft2(float2 *v)
{
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3)
{
    const float2 s0 = cadd(a0, a2), s1 = csub(a0, a2), s2 = cadd(a1, a3), s3 = mul_mi(csub(a1, a3));
    a0 = cadd(s0, s2);
    a2 = csub(s0, s2);
    a1 = cadd(s1, s3);
    a3 = csub(s1, s3);
}

__device__ __forceinline__ void dft8(float2 *v)
{
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    const float h = 0.70710678118654752440f;  // 1/sqrt(2)
    // W8^1 = (1 - i)/sqrt2, W8^2 = -i, W8^3 = (-1 - i)/sqrt2
    const float2 t1 = make_float2((o1.x + o1.y) * h, (o1.y - o1.x) * h);
    const float2 t2 = mul_mi(o2);
    const float2 t3 = make_float2((o3.y - o3.x) * h, -(o3.x + o3.y) * h);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
}

template <int R>
__device__ __forceinline__ void dft(float2 *v)
{
    if (R == 8) {
        dft8(v);
    } else if (R == 4) {
        dft4(v[0], v[1], v[2], v[3]);
    } else {
        dft2(v);
    }
}

// Reads of one Stockham stage (radix R, current span NS, length N): 8 values
// per thread (8/R butterflies), twiddled and transformed, kept in registers.
// All strides are compile-time constants.
template <int N, int NS, int R>
__device__ __forceinline__ void stage_read(const float2 *tile, const float2 *tw, int c, int g,
                                           float2 (&v)[8])
{
    constexpr int TZ = kXTileBytes / 8 / N;
    constexpr int PER = 8 / R;
    constexpr int NB = N / R;
    constexpr int TSTEP = N / (NS * R);  // twiddle index step per k*r
#pragma unroll
    for (int m = 0; m < PER; m++) {
        const int j = g + m * (N / 8);
        const int k = j & (NS - 1);
        float2 w[R];  // w[r] = tw[k * TSTEP * r]
        if (NS > 1) {
            if (R == 8) {
                // three table reads, the other four by products (a few ulp)
                const float2 w1 = tw[k * TSTEP], w2 = tw[2 * k * TSTEP], w4 = tw[4 * k * TSTEP];
                const float2 w3 = cmul(w1, w2);
                w[1] = w1;
                w[2] = w2;
                w[3] = w3;
                w[4] = w4;
                w[5] = cmul(w1, w4);
                w[6] = cmul(w2, w4);
                w[7] = cmul(w3, w4);
            } else {
#pragma unroll
                for (int r = 1; r < R; r++)
                    w[r] = tw[k * TSTEP * r];
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            float2 x = tile[(j + r * NB) * TZ + c];
            if (NS > 1 && r > 0)
                x = cmul(x, w[r]);
            v[m * R + r] = x;
        }
        dft<R>(&v[m * R]);
    }
}

// Output row of value (m, r) of a stage.
template <int N, int NS, int R>
__device__ __forceinline__ int stage_out_row(int g, int m, int r)
{
    const int j = g + m * (N / 8);
    const int k = j & (NS - 1);
    return (j - k) * R + k + r * NS;
}

template <int N, int NS, int R>
__device__ __forceinline__ void stage_write(float2 *tile, int c, int g, const float2 (&v)[8])
{
    constexpr int TZ = kXTileBytes / 8 / N;
    constexpr int PER = 8 / R;
#pragma unroll
    for (int m = 0; m < PER; m++)
#pragma unroll
        for (int r = 0; r < R; r++)
            tile[stage_out_row<N, NS, R>(g, m, r) * TZ + c] = v[m * R + r];
}

template <int N, int NS>
__device__ __forceinline__ void stage(float2 *tile, const float2 *tw, int c, int g, float2 (&v)[8])
{
    stage_read<N, NS, 8>(tile, tw, c, g, v);
    __syncthreads();
    stage_write<N, NS, 8>(tile, c, g, v);
    __syncthreads();
}

template <int N>
struct FftPlan {
    static constexpr int L = N == 64 ? 6 : N == 128 ? 7 : N == 256 ? 8 : N == 512 ? 9 : 10;
    static constexpr int N8 = (L % 3 == 0) ? L / 3 - 1 : L / 3;  // radix-8 stages before the last
    static constexpr int NSL = 1 << (3 * N8);                      // span before the last stage
    static constexpr int RL = N / NSL;                             // last radix: 8, 4 or 2
};

// Every stage but the last written back; the last stage's values left in v.
template <int N>
__device__ __forceinline__ void fft_to_last(float2 *tile, const float2 *tw, int c, int g,
                                            float2 (&v)[8])
{
    using P = FftPlan<N>;
    if constexpr (P::N8 >= 1)
        stage<N, 1>(tile, tw, c, g, v);
    if constexpr (P::N8 >= 2)
        stage<N, 8>(tile, tw, c, g, v);
    if constexpr (P::N8 >= 3)
        stage<N, 64>(tile, tw, c, g, v);
    stage_read<N, P::NSL, P::RL>(tile, tw, c, g, v);
}

// fft_to_last with every input value passed through f(row, value) as the
// first stage (radix 8, span 1, no twiddles) reads it.
template <int N, typename F>
__device__ __forceinline__ void fft_to_last_in(float2 *tile, const float2 *tw, int c, int g,
                                               float2 (&v)[8], F f)
{
    using P = FftPlan<N>;
    static_assert(P::N8 >= 1, "the first stage is radix 8");
    constexpr int TZ = kXTileBytes / 8 / N;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int row = g + r * (N / 8);
        v[r] = f(row, tile[row * TZ + c]);
    }
    dft<8>(v);
    __syncthreads();
    stage_write<N, 1, 8>(tile, c, g, v);
    __syncthreads();
    if constexpr (P::N8 >= 2)
        stage<N, 8>(tile, tw, c, g, v);
    if constexpr (P::N8 >= 3)
        stage<N, 64>(tile, tw, c, g, v);
    stage_read<N, P::NSL, P::RL>(tile, tw, c, g, v);
}

__device__ __forceinline__ int kval_x(int i, int n)
{
    return i <= n / 2 ? i : i - n;
}

__device__ __forceinline__ int bin_of(uint32_t kk2, const uint32_t *thr, int nrb, float bpu_half)
{
    int b = (int)(bpu_half * __logf((float)kk2));
    b = max(0, min(nrb - 1, b));
    while (kk2 >= thr[b + 1])
        b++;
    while (b > 0 && kk2 < thr[b])
        b--;
    return b;
}

// The last stage: write the outputs (natural row order) and, when binning,
// the per-mode values v into vals[c * (N + 1) + row].
template <int N, bool BIN>
__device__ __forceinline__ void last_write(float2 *tile, float *vals, const ColInfo &ci, int c,
                                           int g, const float2 (&v)[8], const float (&iwr)[8])
{
    using P = FftPlan<N>;
    constexpr int TZ = kXTileBytes / 8 / N;
    constexpr int PER = 8 / P::RL;
    const float cw = ci.w * 1.f;
#pragma unroll
    for (int m = 0; m < PER; m++)
#pragma unroll
        for (int r = 0; r < P::RL; r++) {
            const int row = stage_out_row<N, P::NSL, P::RL>(g, m, r);
            const float2 f = v[m * P::RL + r];
            tile[row * TZ + c] = f;
            if (BIN) {
                const float p1 = (iwr[m * P::RL + r] * ci.iwj) * ci.iwz;
                const float p2 = p1 * p1;
                vals[c * (N + 1) + row] = cw * (p2 * p2) * fmaf(f.x, f.x, f.y * f.y);
            }
        }
}

template <int N, int MODE>
__global__ void __launch_bounds__(kXThreads, kXCtasPerSm)
    k_xfft(const __grid_constant__ CUtensorMap map, XParams p, DeviceStatus *st)
{
    constexpr bool BIN = MODE == kXBin, GRAD = MODE == kXGrad;
    constexpr int TZ = kXTileBytes / 8 / N;
    constexpr int BOX = N < 256 ? N : 256;
    constexpr int NBOX = N / BOX;
    extern __shared__ __align__(1024) unsigned char xs[];
    float2 *tiles = reinterpret_cast<float2 *>(xs);  // [2][N][TZ]
    unsigned char *q = xs + 2 * kXTileBytes;
    float2 *tw_s = reinterpret_cast<float2 *>(q);
    q += sizeof(float2) * N;
    float *iw_s = reinterpret_cast<float *>(q);
    q += sizeof(float) * N;
    // [2][TZ]: by tile parity, so that the next tile's column table is written
    // while warps may still walk this tile's (no barrier ends a tile)
    ColInfo *cols2 = reinterpret_cast<ColInfo *>(q);
    q += sizeof(ColInfo) * 2 * TZ;
    float *vals = reinterpret_cast<float *>(q);                  // [TZ][N + 1]
    q += BIN ? sizeof(float) * TZ * (N + 1) : 0;
    q = xs + ((q - xs + 15) & ~(size_t)15);
    float *whist = reinterpret_cast<float *>(q);                 // [warps][nrbins]
    q += BIN ? sizeof(float) * (kXThreads / 32) * p.nrbins : 0;
    q = xs + ((q - xs + 15) & ~(size_t)15);
    double *chist = reinterpret_cast<double *>(q);               // [nrbins]
    q += BIN ? sizeof(double) * p.nrbins : 0;
    uint32_t *thr = reinterpret_cast<uint32_t *>(q);             // [nrbins + 1]
    q += (BIN || GRAD) ? sizeof(uint32_t) * (p.nrbins + 1) : 0;
    float *gco = reinterpret_cast<float *>(q);                   // [nrbins] (GRAD)
    __shared__ __align__(8) unsigned long long bar[2];

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int c = tid % TZ, g = tid / TZ;  // FFT: column and butterfly group
    for (int i = tid; i < N; i += kXThreads) {
        tw_s[i] = p.tw[i];
        iw_s[i] = (BIN || GRAD) ? p.iw[i] : 0.f;
    }
    if (BIN) {
        for (int i = tid; i < (kXThreads / 32) * p.nrbins; i += kXThreads)
            whist[i] = 0.f;
        for (int i = tid; i < p.nrbins; i += kXThreads)
            chist[i] = 0.0;
    }
    if (BIN || GRAD)
        for (int i = tid; i <= p.nrbins; i += kXThreads)
            thr[i] = p.thr[i];
    if (GRAD)
        for (int i = tid; i < p.nrbins; i += kXThreads)
            gco[i] = p.gcoef[i];
    if (tid == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async();
    }
    __syncthreads();
    // Binning each field of a batch: a CTA's tiles run through the fields in
    // order, so its histogram goes out at each field's last tile; fields it
    // has no tile of get zeros (those before its first tile here).
    const int bf = p.bin_fields;
    double *cta_part = (BIN && bf > 1) ? p.partial + (size_t)blockIdx.x * bf * p.nrbins : nullptr;
    if (BIN && bf > 1)
        for (int i = tid; i < ((int)blockIdx.x / p.tiles_per_field) * p.nrbins; i += kXThreads)
            cta_part[i] = 0.0;
    // iw(kx) of the 8 rows this thread's last stage writes: the same in every tile
    float iwr[8];
    {
        using P = FftPlan<N>;
#pragma unroll
        for (int m = 0; m < 8 / P::RL; m++)
#pragma unroll
            for (int r = 0; r < P::RL; r++)
                iwr[m * P::RL + r] = BIN ? iw_s[stage_out_row<N, P::NSL, P::RL>(g, m, r)] : 0.f;
    }

    auto issue = [&](int t, int buf) {
        const int b = t / p.tiles_per_field, f0 = (t - b * p.tiles_per_field) * TZ;
        float2 *dst = tiles + buf * (kXTileBytes / (int)sizeof(float2));
        mbar_expect_tx(&bar[buf], (unsigned)kXTileBytes);
#pragma unroll
        for (int k = 0; k < NBOX; k++)
            tma_load_2d(dst + k * BOX * TZ, &map, 2 * f0, b * N + k * BOX, &bar[buf]);
    };

    unsigned timeouts = 0;
    if (tid == 0 && (int)blockIdx.x < p.ntiles)
        issue(blockIdx.x, 0);
    int k = 0;
    for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x, k++) {
        const int buf = k & 1;
        float2 *tile = tiles + buf * (kXTileBytes / (int)sizeof(float2));
        if (tid == 0 && t + (int)gridDim.x < p.ntiles) {
            bulk_wait_read_all();  // the store from the other buffer has read it
            issue(t + gridDim.x, buf ^ 1);
        }
        const int b = t / p.tiles_per_field, f0 = (t - b * p.tiles_per_field) * TZ;
        if ((BIN || GRAD) && tid < TZ) {
            const int f = f0 + tid;
            ColInfo ci;
            if (f < p.ncols) {
                const int j = f / p.hc, kz = f - j * p.hc;
                const int ky = kval_x(j, N);
                ci.r2 = ky * ky + kz * kz;
                ci.iwj = p.iw[j];
                ci.iwz = p.iw[kz];
                ci.w = (kz == 0 || kz == N / 2) ? 1.f : 2.f;
                ci.special = (j == 0 && kz == 0) ? 1 : (j == N / 2 && kz == N / 2 && p.corner) ? 2 : 0;
                ci.run = kz == 0 ? 1 : 0;
            } else {
                ci.r2 = -1;
                ci.run = 0;
                ci.iwj = ci.iwz = ci.w = 0.f;
                ci.special = 0;
            }
            cols2[(k & 1) * TZ + tid] = ci;
        }
        zero_share<kXThreads>(p.zero, p.zero_units, p.zero_per_tile, t, tid);
        if (!mbar_wait(&bar[buf], (unsigned)(k >> 1) & 1u))
            timeouts++;
        __syncthreads();

        float2 v[8];
        if (GRAD) {
            // H = G_b V_m F_m (c_m / mult_m = 1 for even N), conjugated on the
            // way in; the same bins as the forward binning (thr, iw).
            const ColInfo ci = cols2[(k & 1) * TZ + c];
            auto scale = [&](int row, float2 x) -> float2 {
                const int kx = kval_x(row, N);
                const uint32_t kk2 = (uint32_t)(kx * kx) + (uint32_t)ci.r2;
                if (ci.r2 < 0 || kk2 == 0)
                    return make_float2(0.f, 0.f);
                int bb = (int)(p.bpu_half * __logf((float)kk2));
                bb = max(0, min(p.nrbins - 1, bb));
                while (bb + 1 < p.nrbins && kk2 >= thr[bb + 1])
                    bb++;
                while (bb > 0 && kk2 < thr[bb])
                    bb--;
                const float pz = (iw_s[row] * ci.iwj) * ci.iwz;
                const float p2 = pz * pz;
                const float s = gco[bb] * (p2 * p2);
                return make_float2(s * x.x, -(s * x.y));
            };
            fft_to_last_in<N>(tile, tw_s, c, g, v, scale);
#pragma unroll
            for (int r = 0; r < 8; r++)
                v[r].y = -v[r].y;
        } else {
            fft_to_last<N>(tile, tw_s, c, g, v);
        }
        __syncthreads();
        const ColInfo *cols = cols2 + (k & 1) * TZ;
        const ColInfo ci = BIN ? cols[c] : ColInfo{};
        last_write<N, BIN>(tile, vals, ci, c, g, v, iwr);
        if (BIN && ci.special) {
            // the skipped k = 0 mode and the exact corner mode
            const int row = ci.special == 1 ? 0 : N / 2;
            const float p1 = (iw_s[row] * ci.iwj) * ci.iwz;
            const float p2 = p1 * p1;
            const float cv = ci.special == 2 ? (float)p.corner[bf > 1 ? b : 0] : 0.f;
            const float pw = ci.special == 1 ? 0.f : cv * cv;
            if (g == 0)  // one thread of the column writes it
                vals[c * (N + 1) + row] = ci.w * (p2 * p2) * pw;
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
#pragma unroll
            for (int kb = 0; kb < NBOX; kb++)
                tma_store_2d(&map, 2 * f0, b * N + kb * BOX, tile + kb * BOX * TZ);
            bulk_commit();
        }

        if (BIN) {
            // Walk columns of a row with a running bin: 8 modes per thread
            // (8 columns of one row; for N = 1024, 4 columns of two rows).
            // The column structure is the same for every lane of a warp (lanes
            // differ in the row): the bin is looked up where a run of
            // consecutive kz starts (the first column, or kz = 0 of a new ky),
            // so those lookups are warp-uniform; along a run |k|^2 grows and
            // the bin only steps up past the next threshold.
            constexpr int ROWS_PT = N > kXThreads ? N / kXThreads : 1;
            constexpr int COLS_PT = (kXTileBytes / 8 / kXThreads) / ROWS_PT;
#pragma unroll
            for (int rr = 0; rr < ROWS_PT; rr++) {
                const int row = N > kXThreads ? tid + rr * kXThreads : tid % N;
                const int c0 = N > kXThreads ? 0 : (tid / N) * COLS_PT;
                const int kx = kval_x(row, N);
                const uint32_t kx2 = (uint32_t)(kx * kx);
                int cb = p.nrbins;  // sentinel: no mode yet
                uint32_t nx = 0;    // the open bin's upper threshold
                float acc = 0.f;
#pragma unroll
                for (int cc = 0; cc < COLS_PT; cc++) {
                    const int r2 = cols[c0 + cc].r2;
                    if (r2 < 0)
                        break;  // padding columns: only after the field's last column
                    const uint32_t kk2 = kx2 + (uint32_t)r2;
                    if (cc == 0 || cols[c0 + cc].run) {
                        if (cb < p.nrbins)
                            atomicAdd(&whist[wid * p.nrbins + cb], acc);
                        cb = bin_of(kk2, thr, p.nrbins, p.bpu_half);
                        nx = thr[cb + 1];
                        acc = 0.f;
                    } else {
                        while (kk2 >= nx) {  // thr[nrbins] = 2^32 - 1 ends it
                            atomicAdd(&whist[wid * p.nrbins + cb], acc);
                            acc = 0.f;
                            cb++;
                            nx = thr[cb + 1];
                        }
                    }
                    acc += vals[(c0 + cc) * (N + 1) + row];
                }
                // Segmented scan over the lanes' open bins (the warp's rows lie
                // in one half of the axis, so the bins are monotone across it).
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int ku = __shfl_up_sync(0xffffffffu, cb, o);
                    const float x = __shfl_up_sync(0xffffffffu, acc, o);
                    if (lane >= o && ku == cb)
                        acc += x;
                }
                const int kd = __shfl_down_sync(0xffffffffu, cb, 1);
                if (cb < p.nrbins && (lane == 31 || kd != cb))
                    atomicAdd(&whist[wid * p.nrbins + cb], acc);
            }
            // The warps' FP32 histograms go into the CTA's FP64 one every 8
            // tiles and after the CTA's last tile of a binned field (the
            // condition is uniform); a field's histogram then goes out.
            const int tn = t + (int)gridDim.x;
            const int bn = tn < p.ntiles ? tn / p.tiles_per_field : -1;  // -1: no next tile
            const bool field_end = bn != b && (bf > 1 || bn < 0);
            if ((k & 7) == 7 || field_end) {
                __syncthreads();
                for (int bb = tid; bb < p.nrbins; bb += kXThreads) {
                    float s = 0.f;
                    for (int w = 0; w < kXThreads / 32; w++) {
                        s += whist[w * p.nrbins + bb];
                        whist[w * p.nrbins + bb] = 0.f;
                    }
                    chist[bb] += (double)s;
                    if (bf > 1 && field_end) {
                        cta_part[(size_t)b * p.nrbins + bb] = chist[bb];
                        chist[bb] = 0.0;
                    }
                }
                if (bf > 1 && field_end) {  // fields up to the next tile's get zeros
                    const int upto = bn < 0 ? bf : bn;
                    for (int i = tid; i < (upto - b - 1) * p.nrbins; i += kXThreads)
                        cta_part[(size_t)(b + 1) * p.nrbins + i] = 0.0;
                }
            }
        }
    }
    if (tid == 0)
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // stores complete
    if (BIN && bf == 1) {
        __syncthreads();
        for (int bb = tid; bb < p.nrbins; bb += kXThreads)
            p.partial[(size_t)blockIdx.x * p.nrbins + bb] = chist[bb];
    }
    timeouts = __reduce_add_sync(0xffffffffu, timeouts);
    if (lane == 0 && timeouts)
        atomicAdd(&st->timeouts, (unsigned long long)timeouts);
}

// ---- z and y passes of the forward transform (64 <= N <= 512, powers of two)
//
// k_zfft: the length-N real-to-complex transform of every z row, one warp per
// row.  The row's N reals become M = N/2 complex values z[n] = x[2n] +
// i x[2n+1]; an M-point FFT with n = lane + 32 m (R = M/32 values per lane):
//   1. an R-point DFT over m in registers, twiddles W_M^{lane k1};
//   2. the 32-point DFTs over lanes, one per k1: for R = 8, a shared-memory
//      exchange gives the four lanes 4 k1 + q the values of l = q + 4 i
//      (i = 0..7); an 8-point DFT over i in registers, twiddles W_32^{q ki},
//      a 4-point DFT across those four lanes (two shuffle stages).  For
//      R < 8, five radix-2 shuffle stages across the warp;
//   3. X[k] = E[k] + W_N^k O[k], k = 0..M, with E = (Z[k] + conj Z[M-k]) / 2
//      and O = (Z[k] - conj Z[M-k]) / 2i.
// The input is the window engine's 64-bit accumulator, converted as
// k_window_convert does (accumulator minus the fixed-point mean, rounded
// once), so that pass is skipped; the output is the FP32 grid's row.  Rows are
// prefetched one row ahead by 16-byte asynchronous copies into a per-warp
// buffer; each lane copies and later reads only its own chunks, so the buffer
// needs no warp synchronisation.
constexpr int kZThreads = 256;

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}

__device__ __forceinline__ int zpad(int i)
{
    return i + (i >> 5);
}

// Radix-2 decimation-in-frequency step across lanes xor s (upper lanes take
// (a - b) W, lower lanes a + b).
__device__ __forceinline__ float2 dif_shfl(float2 v, int s, bool upper, float2 w)
{
    const float2 q = make_float2(__shfl_xor_sync(0xffffffffu, v.x, s),
                                 __shfl_xor_sync(0xffffffffu, v.y, s));
    return upper ? cmul(csub(q, v), w) : cadd(v, q);
}

template <int N>
__global__ void __launch_bounds__(kZThreads)
    k_zfft(const unsigned long long *__restrict__ acc, float *grid, int64_t nrows,
           int row_floats, const float2 *__restrict__ tw_g, const DeviceStatus *__restrict__ st)
{
    constexpr int M = N / 2;
    constexpr int R = M / 32;
    __shared__ float2 tw[N];
    __shared__ float2 zs_all[kZThreads / 32][M + M / 32];  // Z[k] (or exchange) at zpad(k)
    extern __shared__ __align__(16) unsigned char zdyn[];  // [warps][M] longlong2
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        tw[i] = tw_g[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float2 *zs = zs_all[wid];
    longlong2 *pre = reinterpret_cast<longlong2 *>(zdyn) + wid * M;
    auto prefetch = [&](int64_t r) {
        const longlong2 *src = reinterpret_cast<const longlong2 *>(acc + (size_t)r * row_floats);
#pragma unroll
        for (int m = 0; m < R; m++)
            cp_async16(pre + lane + 32 * m, src + lane + 32 * m);
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    const long long mean = st->mean_fixed;
    const float inv_scale = ldexpf(1.f, -st->fx_shift);
    const int br = (int)(__brev((unsigned)lane) >> 27);
    const int k1g = lane >> 2, qg = lane & 3;                   // R = 8: group and member
    const int qrev = ((qg & 1) << 1) | (qg >> 1);               // 2-bit reversal
    const int64_t nw = (int64_t)gridDim.x * (kZThreads / 32);
    const int64_t row0 = (int64_t)blockIdx.x * (kZThreads / 32) + wid;
    if (row0 < nrows)
        prefetch(row0);
    for (int64_t row = row0; row < nrows; row += nw) {
        const size_t base = (size_t)row * (size_t)row_floats;
        float2 v[R];
        asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
        for (int m = 0; m < R; m++) {
            const longlong2 a = pre[lane + 32 * m];
            v[m] = make_float2(i64_to_f32_rn(a.x - mean) * inv_scale,
                               i64_to_f32_rn(a.y - mean) * inv_scale);
        }
        // the values are in registers: this lane's chunks of the buffer are free
        if (row + nw < nrows)
            prefetch(row + nw);
        if constexpr (R > 1)
            dft<R>(v);
#pragma unroll
        for (int k1 = 1; k1 < R; k1++)
            v[k1] = cmul(v[k1], tw[(2 * lane * k1) & (N - 1)]);
        if constexpr (R == 8) {
            // exchange: y_l[k1] at (k1, l) -> lane 4 k1 + q takes l = q + 4 i
#pragma unroll
            for (int k1 = 0; k1 < 8; k1++)
                zs[zpad(k1 * 32 + lane)] = v[k1];
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 8; i++)
                v[i] = zs[zpad(k1g * 32 + qg + 4 * i)];
            __syncwarp();
            dft8(v);
#pragma unroll
            for (int ki = 1; ki < 8; ki++)
                v[ki] = cmul(v[ki], tw[(qg * ki * (N / 32)) & (N - 1)]);  // W_32^{q ki}
            // 4-point DFT over q across the lanes of the group (xor 2, then xor 1)
            const float2 w2 = tw[(qg & 1) * (N / 4)];  // W_4^{q mod 2}
#pragma unroll
            for (int ki = 0; ki < 8; ki++) {
                v[ki] = dif_shfl(v[ki], 2, (qg & 2) != 0, w2);
                v[ki] = dif_shfl(v[ki], 1, (qg & 1) != 0, make_float2(1.f, 0.f));
            }
            // lane holds Z[k1 + 8 (ki + 8 bitrev2(q))]
#pragma unroll
            for (int ki = 0; ki < 8; ki++)
                zs[zpad(k1g + 8 * (ki + 8 * qrev))] = v[ki];
        } else {
#pragma unroll
            for (int s = 16; s >= 1; s >>= 1) {
                const bool upper = (lane & s) != 0;
                const float2 w = tw[(lane & (s - 1)) * (N / (2 * s))];  // W_{2s}^{lane mod s}
#pragma unroll
                for (int k1 = 0; k1 < R; k1++)
                    v[k1] = dif_shfl(v[k1], s, upper, w);
            }
            // lane holds Z[k1 + R bitrev5(lane)]
#pragma unroll
            for (int k1 = 0; k1 < R; k1++)
                zs[zpad(k1 + R * br)] = v[k1];
        }
        __syncwarp();
        float2 *out = reinterpret_cast<float2 *>(grid + base);
#pragma unroll
        for (int j = 0; j <= R; j++) {
            const int k = lane + 32 * j;
            if (k <= M) {
                const int ka = k == M ? 0 : k;      // Z[N/2] = Z[0]
                const int kb = k == 0 ? 0 : M - k;  // Z[(N/2 - k) mod N/2]
                const float2 a = zs[zpad(ka)], b = zs[zpad(kb)];
                const float2 e = make_float2(a.x + b.x, a.y - b.y);
                const float2 o = make_float2(a.x - b.x, a.y + b.y);
                const float2 wo = cmul(tw[k], o);
                out[k] = make_float2(0.5f * (e.x + wo.y), 0.5f * (e.y - wo.x));
            }
        }
        __syncwarp();
    }
}

// ---- the z pass for N = 1024, written kz-major --------------------------------
//
// At N = 1024 the y and x transforms run as one batched 2-D cuFFT C2C over
// contiguous N x N planes, one per kz (3.0 ms at 1024^3, against 5.4 ms for
// the in-place 3-D R2C), so this z pass writes its output kz-major: the
// transform of row (x, y) at kz goes to S[kz][x][y], S holding N/2+1 planes of
// N x N complex values in the grid's memory.  One CTA takes kTRows
// consecutive rows (one x, consecutive y), one warp per row:
//   1. the row's N accumulator values, converted as k_window_convert converts
//      them (minus the fixed-point mean, rounded once), as M = N/2 complex
//      values z[n] = x[2n] + i x[2n+1], lane l holding n = l + 32 m (m < 16);
//   2. a 16-point DFT over m in registers, twiddles W_M^{l k1};
//   3. the 32-point DFTs over the lanes, one per k1: a shared-memory exchange
//      gives lanes 2 k1 and 2 k1 + 1 the values l = q + 2 i (i < 16), a
//      16-point DFT over i, twiddles W_32^{q ki}, then a 2-point DFT across
//      the lane pair, so that lane (k1, q) holds Z[k1 + 16 (ki + 16 q)];
//   4. X[k] = E[k] + W_N^k O[k], k = 0..M, into a [kz][row] shared buffer;
//   5. the CTA's rows leave as runs of kTRows consecutive y per kz.
// The accumulator is left as it is: the kz-major binning pass clears it.
constexpr int kTRows = 16;  // rows per CTA: 128-byte runs per kz plane (8: 3.54 -> 3.41 ms)
constexpr int kTThreads = kTRows * 32;

// Forward 16-point DFT in registers (two 8-point DFTs and W_16 twiddles).
__device__ __forceinline__ void dft16(float2 *v)
{
    float2 e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
    }
    dft8(e);
    dft8(o);
    // W_16^k = cos(pi k / 8) - i sin(pi k / 8), k = 0..7
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float h = 0.70710678118654752440f;
    const float2 w[8] = {make_float2(1.f, 0.f),  make_float2(c1, -s1), make_float2(h, -h),
                         make_float2(s1, -c1),   make_float2(0.f, -1.f), make_float2(-s1, -c1),
                         make_float2(-h, -h),    make_float2(-c1, -s1)};
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float2 t = k == 0 ? o[0] : cmul(o[k], w[k]);
        v[k] = cadd(e[k], t);
        v[k + 8] = csub(e[k], t);
    }
}

__global__ void __launch_bounds__(kTThreads)
    k_zfft_t1024(const unsigned long long *__restrict__ acc, float2 *__restrict__ spec, int row_floats,
                 const float2 *__restrict__ tw, const DeviceStatus *__restrict__ st)
{
    constexpr int N = 1024, M = N / 2, R = M / 32, HC = N / 2 + 1;
    extern __shared__ __align__(16) unsigned char ts[];
    float2 *zx = reinterpret_cast<float2 *>(ts) + (threadIdx.x >> 5) * (M + M / 32);
    float2 *tb = reinterpret_cast<float2 *>(ts) + kTRows * (M + M / 32);  // [HC][kTRows + 1]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * kTRows;
    const int x = (int)(row0 / N), y0 = (int)(row0 - (int64_t)x * N);
    const long long mean = st->mean_fixed;
    const float inv_scale = ldexpf(1.f, -st->fx_shift);

    const longlong2 *src =
        reinterpret_cast<const longlong2 *>(acc + (size_t)(row0 + wid) * (size_t)row_floats);
    longlong2 a[R];
#pragma unroll
    for (int m = 0; m < R; m++)
        a[m] = src[lane + 32 * m];
    float2 v[R];
#pragma unroll
    for (int m = 0; m < R; m++)
        v[m] = make_float2(i64_to_f32_rn(a[m].x - mean) * inv_scale,
                           i64_to_f32_rn(a[m].y - mean) * inv_scale);

    dft16(v);
#pragma unroll
    for (int k1 = 1; k1 < R; k1++)
        v[k1] = cmul(v[k1], __ldg(tw + ((2 * lane * k1) & (N - 1))));  // W_M^{l k1}
#pragma unroll
    for (int k1 = 0; k1 < R; k1++)
        zx[zpad(k1 * 32 + lane)] = v[k1];
    __syncwarp();
    const int k1g = lane >> 1, q = lane & 1;
#pragma unroll
    for (int i = 0; i < R; i++)
        v[i] = zx[zpad(k1g * 32 + q + 2 * i)];
    __syncwarp();
    dft16(v);
    if (q) {
#pragma unroll
        for (int ki = 1; ki < R; ki++)
            v[ki] = cmul(v[ki], __ldg(tw + ((N / 32) * ki)));  // W_32^{ki}
    }
#pragma unroll
    for (int ki = 0; ki < R; ki++)
        v[ki] = dif_shfl(v[ki], 1, q != 0, make_float2(1.f, 0.f));
#pragma unroll
    for (int ki = 0; ki < R; ki++)
        zx[zpad(k1g + 16 * (ki + 16 * q))] = v[ki];
    __syncwarp();
#pragma unroll
    for (int j = 0; j <= R; j++) {
        const int k = lane + 32 * j;
        if (k <= M) {
            const int ka = k == M ? 0 : k;      // Z[N/2] = Z[0]
            const int kb = k == 0 ? 0 : M - k;  // Z[(N/2 - k) mod N/2]
            const float2 za = zx[zpad(ka)], zb = zx[zpad(kb)];
            const float2 e = make_float2(za.x + zb.x, za.y - zb.y);
            const float2 o = make_float2(za.x - zb.x, za.y + zb.y);
            const float2 wo = cmul(__ldg(tw + k), o);
            tb[k * (kTRows + 1) + wid] = make_float2(0.5f * (e.x + wo.y), 0.5f * (e.y - wo.x));
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < HC * kTRows; e += kTThreads) {
        const int kz = e / kTRows, r = e - kz * kTRows;
        spec[((size_t)kz * N + (size_t)x) * N + (size_t)(y0 + r)] = tb[kz * (kTRows + 1) + r];
    }
}

// The adjoint's inverse z pass for N = 1024 (the transpose of k_zfft_t1024's
// job): after the mode gradient and an inverse batched 2-D C2C over the kz
// planes, the kz-major array holds, for every row (x, y), the N/2+1 values
// X[kz] whose unnormalised C2R along z is that row of dL/drho.  One CTA takes
// kTRows consecutive rows: their X[kz] come in as runs of kTRows consecutive y
// per kz into a [kz][row] shared buffer; then per row (one warp)
//   Z[k] = (X[k] + conj X[M-k]) + i W_N^{-k} (X[k] - conj X[M-k]),  k < M,
// (Im X[0] and Im X[M] dropped, as a real transform drops them), and the
// unnormalised inverse M-point DFT of Z, as conj(DFT(conj Z)) with the
// forward pass's structure, gives x[2n] + i x[2n+1] = z[n]: the real row,
// written to `out` in the padded row layout (row_floats floats per row).
__global__ void __launch_bounds__(kTThreads)
    k_zifft_t1024(const float2 *__restrict__ spec, float *__restrict__ out, int row_floats,
                  const float2 *__restrict__ tw)
{
    constexpr int N = 1024, M = N / 2, R = M / 32, HC = N / 2 + 1;
    extern __shared__ __align__(16) unsigned char ts[];
    float2 *zx = reinterpret_cast<float2 *>(ts) + (threadIdx.x >> 5) * (M + M / 32);
    float2 *tb = reinterpret_cast<float2 *>(ts) + kTRows * (M + M / 32);  // [HC][kTRows + 1]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * kTRows;
    const int x = (int)(row0 / N), y0 = (int)(row0 - (int64_t)x * N);
    {
        // every load of this thread in flight before any store (the runs are
        // kTRows values of one kz plane, planes N^2 values apart)
        constexpr int PER = (HC * kTRows + kTThreads - 1) / kTThreads;
        float2 in[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int e = threadIdx.x + i * kTThreads;
            const int kz = e / kTRows, r = e - kz * kTRows;
            in[i] = e < HC * kTRows
                        ? __ldg(spec + ((size_t)kz * N + (size_t)x) * N + (size_t)(y0 + r))
                        : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int e = threadIdx.x + i * kTThreads;
            const int kz = e / kTRows, r = e - kz * kTRows;
            if (e < HC * kTRows)
                tb[kz * (kTRows + 1) + r] = in[i];
        }
    }
    __syncthreads();
    float2 v[R];
#pragma unroll
    for (int m = 0; m < R; m++) {
        const int k = lane + 32 * m;
        float2 a = tb[k * (kTRows + 1) + wid], b = tb[(M - k) * (kTRows + 1) + wid];
        if (k == 0) {
            a.y = 0.f;
            b.y = 0.f;
        }
        const float2 s = make_float2(a.x + b.x, a.y - b.y);  // X[k] + conj X[M-k]
        const float2 d = make_float2(a.x - b.x, a.y + b.y);  // X[k] - conj X[M-k]
        const float2 w = __ldg(tw + k);
        const float2 wd = cmul(make_float2(w.x, -w.y), d);   // W_N^{-k} d
        v[m] = make_float2(s.x - wd.y, -(s.y + wd.x));       // conj(s + i wd)
    }
    dft16(v);
#pragma unroll
    for (int k1 = 1; k1 < R; k1++)
        v[k1] = cmul(v[k1], __ldg(tw + ((2 * lane * k1) & (N - 1))));
#pragma unroll
    for (int k1 = 0; k1 < R; k1++)
        zx[zpad(k1 * 32 + lane)] = v[k1];
    __syncwarp();
    const int k1g = lane >> 1, q = lane & 1;
#pragma unroll
    for (int i = 0; i < R; i++)
        v[i] = zx[zpad(k1g * 32 + q + 2 * i)];
    __syncwarp();
    dft16(v);
    if (q) {
#pragma unroll
        for (int ki = 1; ki < R; ki++)
            v[ki] = cmul(v[ki], __ldg(tw + ((N / 32) * ki)));
    }
#pragma unroll
    for (int ki = 0; ki < R; ki++)
        v[ki] = dif_shfl(v[ki], 1, q != 0, make_float2(1.f, 0.f));
#pragma unroll
    for (int ki = 0; ki < R; ki++)
        zx[zpad(k1g + 16 * (ki + 16 * q))] = make_float2(v[ki].x, -v[ki].y);  // conj: z[n]
    __syncwarp();
    float2 *orow = reinterpret_cast<float2 *>(out + (size_t)(row0 + wid) * (size_t)row_floats);
#pragma unroll
    for (int j = 0; j < R; j++) {
        const int nn = lane + 32 * j;
        orow[nn] = zx[zpad(nn)];
    }
}

// kz-major spectrum S[kz][x][y] -> the in-place r2c layout F[x][y][kz] (rows
// of N/2+1 complex values), out of place: 32 x 32 tiles of (kz, y) for one x
// through shared memory, reads coalesced along y, writes along kz.
__global__ void __launch_bounds__(256)
    k_kz_to_rows(const float2 *__restrict__ s, float2 *__restrict__ f, int n, int hc)
{
    __shared__ float2 t[32][33];
    const int x = blockIdx.z;
    const int y0 = blockIdx.x * 32, kz0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int j = ty; j < 32; j += 8) {
        const int kz = kz0 + j, y = y0 + tx;
        if (kz < hc && y < n)
            t[j][tx] = s[((size_t)kz * n + x) * n + y];
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int y = y0 + j, kz = kz0 + tx;
        if (kz < hc && y < n)
            f[((size_t)x * n + y) * hc + kz] = t[tx][j];
    }
}

// k_yfft: the length-N complex transform along y of every (x-plane, kz)
// column, in place in the in-place r2c layout.  Tiles of N rows x TZ columns
// (consecutive kz of one x-plane) are copied into shared memory by 8-byte
// asynchronous copies (cp.async; the rows are (N/2+1)*8 bytes apart, which
// tensor copies cannot address), double-buffered so the next tile streams in
// while this one is transformed by the x pass's Stockham stages; the last
// stage writes straight back.  Columns past kz = N/2 are zero-filled.  (A third
// buffer for the stages to alternate between, halving the barriers, made the
// pass slower: 100 KB of shared memory per CTA leaves the 8-byte copies, which
// go through L1, too little of it.)
__device__ __forceinline__ void cp_async8(void *dst, const void *src, unsigned src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}

template <int N>
__global__ void __launch_bounds__(kXThreads, kXCtasPerSm)
    k_yfft(float2 *spec, int hc, int tiles_per_plane, int64_t ntiles,
           const float2 *__restrict__ tw_g)
{
    constexpr int TZ = kXTileBytes / 8 / N;
    using P = FftPlan<N>;
    extern __shared__ __align__(16) unsigned char ys[];
    float2 *tiles = reinterpret_cast<float2 *>(ys);                   // [2][N][TZ]
    float2 *tw_s = reinterpret_cast<float2 *>(ys + 2 * kXTileBytes);  // [N]
    const int tid = threadIdx.x;
    const int c = tid % TZ, g = tid / TZ;
    for (int i = tid; i < N; i += kXThreads)
        tw_s[i] = tw_g[i];
    auto fetch = [&](int64_t t, float2 *dst) {
        const int64_t plane = t / tiles_per_plane;
        const int kz0 = (int)(t - plane * tiles_per_plane) * TZ;
        const float2 *pl = spec + (size_t)plane * (size_t)N * (size_t)hc;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int e = tid + kXThreads * q;
            const int row = e / TZ, col = e - row * TZ;
            const int kz = kz0 + col;
            const bool in = kz < hc;
            cp_async8(dst + row * TZ + col, pl + (size_t)row * hc + (in ? kz : 0), in ? 8u : 0u);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int k = 0;
    if ((int64_t)blockIdx.x < ntiles)
        fetch(blockIdx.x, tiles);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, k++) {
        float2 *tile = tiles + (k & 1) * (kXTileBytes / (int)sizeof(float2));
        __syncthreads();  // every thread is done with the other buffer
        const bool next = t + gridDim.x < ntiles;
        if (next)
            fetch(t + gridDim.x, tiles + ((k + 1) & 1) * (kXTileBytes / (int)sizeof(float2)));
        if (next)
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        else
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // this tile's copies, from every thread, have landed
        const int64_t plane = t / tiles_per_plane;
        const int kz0 = (int)(t - plane * tiles_per_plane) * TZ;
        float2 *pl = spec + (size_t)plane * (size_t)N * (size_t)hc;
        float2 v[8];
        fft_to_last<N>(tile, tw_s, c, g, v);
        const int kz = kz0 + c;
        if (kz < hc) {
#pragma unroll
            for (int m = 0; m < 8 / P::RL; m++)
#pragma unroll
                for (int r = 0; r < P::RL; r++)
                    pl[(size_t)stage_out_row<N, P::NSL, P::RL>(g, m, r) * hc + kz] =
                        v[m * P::RL + r];
        }
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)f;
        else
            cudaGetLastError();
    });
    return fn;
}

int xfft_tz(int dims)
{
    return kXTileBytes / 8 / dims;
}

size_t xfft_smem(int dims, int nrbins, int mode)
{
    const int tz = xfft_tz(dims);
    size_t s = 2 * (size_t)kXTileBytes + sizeof(float2) * dims + sizeof(float) * dims +
               sizeof(ColInfo) * 2 * tz;
    if (mode == kXBin) {
        s += sizeof(float) * tz * (dims + 1);
        s = (s + 15) & ~(size_t)15;
        s += sizeof(float) * (kXThreads / 32) * nrbins;
        s = (s + 15) & ~(size_t)15;
        s += sizeof(double) * nrbins + sizeof(uint32_t) * (nrbins + 1);
    } else if (mode == kXGrad) {
        // the kernel's empty binning buffers still round the offset up to 16
        s = (s + 15) & ~(size_t)15;
        s += sizeof(uint32_t) * (nrbins + 1) + sizeof(float) * nrbins;
    }
    return s;
}

}  // namespace

// Used for N <= 512: at N = 1024 the tile is 4 columns wide (32-byte rows)
// and the 3-D cuFFT + binning path was faster (6.6 ms against 10.3 ms).
bool xfft_supported(int dims)
{
    return dims >= 64 && dims <= 512 && (dims & (dims - 1)) == 0 && encode_fn() != nullptr;
}

bool xfft_grad_supported(int dims, int nrbins)
{
    return xfft_supported(dims) && nrbins >= 1 && xfft_smem(dims, nrbins, kXGrad) <= 227 * 1024;
}

bool xfft_bin_supported(int dims, int nrbins)
{
    return xfft_supported(dims) && nrbins >= 1 && nrbins <= kXMaxBins &&
           xfft_smem(dims, nrbins, kXBin) <= 227 * 1024;
}

void xfft_twiddles(int dims, std::vector<float> *out)
{
    out->resize(2 * (size_t)dims);
    const double pi = 3.14159265358979323846;
    for (int m = 0; m < dims; m++) {
        const double a = -2.0 * pi * (double)m / (double)dims;
        (*out)[2 * (size_t)m] = (float)std::cos(a);
        (*out)[2 * (size_t)m + 1] = (float)std::sin(a);
    }
}

namespace {

cudaError_t launch_xfft(const GridGeom &g, float *grids, int nbatch, const float2 *tw, int mode,
                        const XfftBin *bin, const XfftGrad *grad, void *zero, int64_t zero_bytes,
                        int num_sms, DeviceStatus *dstat, cudaStream_t stream, int64_t *launches)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc)
        return cudaErrorNotSupported;
    const int n = g.dims;
    XParams p;
    p.dims = n;
    p.hc = g.hc;
    p.tz = xfft_tz(n);
    {
        int l = 0;
        while ((1 << l) < n)
            l++;
        p.log2n = l;
        p.n8 = (l % 3 == 0) ? l / 3 - 1 : l / 3;  // the last stage is read separately
    }
    p.ncols = n * g.hc;
    p.tiles_per_field = (p.ncols + p.tz - 1) / p.tz;
    p.ntiles = p.tiles_per_field * nbatch;
    p.box_rows = std::min(n, 256);
    p.tw = tw;
    p.nrbins = bin ? bin->nrbins : grad ? grad->nrbins : 0;
    p.bpu_half = bin ? bin->bpu_half : grad ? grad->bpu_half : 0.f;
    p.thr = bin ? bin->thr : grad ? grad->thr : nullptr;
    p.iw = bin ? bin->iw : grad ? grad->iw : nullptr;
    p.corner = bin ? bin->corner : nullptr;
    p.partial = bin ? bin->partial : nullptr;
    p.bin_fields = bin ? bin->fields : 1;
    if (bin && bin->fields != 1 && bin->fields != nbatch)
        return cudaErrorInvalidValue;
    p.gcoef = grad ? grad->gcoef : nullptr;
    p.zero = zero_bytes > 0 ? static_cast<uint4 *>(zero) : nullptr;
    p.zero_units = zero_bytes / 16;
    p.zero_per_tile = (p.zero_units + p.ntiles - 1) / p.ntiles;

    CUtensorMap map;
    const cuuint64_t gdim[2] = {(cuuint64_t)2 * p.ncols, (cuuint64_t)n * nbatch};
    const cuuint64_t gstride[1] = {(cuuint64_t)p.ncols * 8};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * p.tz), (cuuint32_t)p.box_rows};
    const cuuint32_t estride[2] = {1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, grids, gdim, gstride, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const int ctas = std::min(p.ntiles, num_sms * kXCtasPerSm);
    const size_t smem = xfft_smem(n, p.nrbins, mode);
    void (*kern)(const CUtensorMap, XParams, DeviceStatus *) = nullptr;
#define GENPK_XFFT_PICK(NN)                                                           \
    case NN:                                                                          \
        kern = mode == kXBin ? k_xfft<NN, kXBin>                                      \
                             : mode == kXGrad ? k_xfft<NN, kXGrad> : k_xfft<NN, kXPlain>; \
        break;
    switch (n) {
        GENPK_XFFT_PICK(64)
        GENPK_XFFT_PICK(128)
        GENPK_XFFT_PICK(256)
        GENPK_XFFT_PICK(512)
        GENPK_XFFT_PICK(1024)
    default:
        return cudaErrorNotSupported;
    }
#undef GENPK_XFFT_PICK
    cudaError_t err;
    if ((err = ensure_dynamic_smem(kern, smem)) != cudaSuccess)
        return err;
    kern<<<ctas, kXThreads, smem, stream>>>(map, p, dstat);
    (*launches)++;
    return cudaGetLastError();
}

}  // namespace

cudaError_t xfft_pass(const GridGeom &g, float *grids, int nbatch, const float2 *tw,
                      const XfftBin *bin, void *zero, int64_t zero_bytes, int num_sms,
                      DeviceStatus *dstat, cudaStream_t stream, int64_t *launches)
{
    return launch_xfft(g, grids, nbatch, tw, bin ? kXBin : kXPlain, bin, nullptr, zero,
                       zero_bytes, num_sms, dstat, stream, launches);
}

cudaError_t xfft_grad_pass(const GridGeom &g, float *grid, const float2 *tw, const XfftGrad &grad,
                           int num_sms, DeviceStatus *dstat, cudaStream_t stream,
                           int64_t *launches)
{
    return launch_xfft(g, grid, 1, tw, kXGrad, nullptr, &grad, nullptr, 0, num_sms, dstat, stream,
                       launches);
}

cudaError_t zfft_pass(const GridGeom &g, float *grid, const unsigned long long *acc,
                      const float2 *tw, const DeviceStatus *dstat, int num_sms,
                      cudaStream_t stream, int64_t *launches)
{
    const int n = g.dims;
    const int64_t nrows = (int64_t)n * n;
    const int ctas = (int)std::min<int64_t>((nrows + 7) / 8, (int64_t)num_sms * 8);
    // prefetch buffers of the accumulator rows: one row per warp
    const int pre = (int)(sizeof(longlong2) * (kZThreads / 32) * (n / 2));
    void (*kern)(const unsigned long long *, float *, int64_t, int, const float2 *,
                 const DeviceStatus *) = nullptr;
    switch (n) {
    case 64:
        kern = k_zfft<64>;
        break;
    case 128:
        kern = k_zfft<128>;
        break;
    case 256:
        kern = k_zfft<256>;
        break;
    case 512:
        kern = k_zfft<512>;
        break;
    default:
        return cudaErrorNotSupported;
    }
    cudaError_t err;
    if ((err = ensure_dynamic_smem(kern, (size_t)pre)) != cudaSuccess)
        return err;
    kern<<<ctas, kZThreads, pre, stream>>>(acc, grid, nrows, g.row, tw, dstat);
    (*launches)++;
    return cudaGetLastError();
}

bool zfft_kz_supported(int dims)
{
    return dims == 1024;
}

cudaError_t zfft_kz_pass(const GridGeom &g, float *grid, const unsigned long long *acc, const float2 *tw,
                         const DeviceStatus *dstat, cudaStream_t stream, int64_t *launches)
{
    if (g.dims != 1024)
        return cudaErrorNotSupported;
    constexpr int M = 512, HC = 513;
    const size_t smem = sizeof(float2) * ((size_t)kTRows * (M + M / 32) + (size_t)HC * (kTRows + 1));
    cudaError_t err;
    if ((err = ensure_dynamic_smem(k_zfft_t1024, smem)) != cudaSuccess)
        return err;
    const int64_t nrows = (int64_t)g.dims * g.dims;
    k_zfft_t1024<<<(unsigned)(nrows / kTRows), kTThreads, smem, stream>>>(
        acc, reinterpret_cast<float2 *>(grid), g.row, tw, dstat);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t zifft_kz_pass(const GridGeom &g, const float *kz_major, float *out, const float2 *tw,
                          cudaStream_t stream, int64_t *launches)
{
    if (g.dims != 1024)
        return cudaErrorNotSupported;
    constexpr int M = 512, HC = 513;
    const size_t smem = sizeof(float2) * ((size_t)kTRows * (M + M / 32) + (size_t)HC * (kTRows + 1));
    cudaError_t err;
    if ((err = ensure_dynamic_smem(k_zifft_t1024, smem)) != cudaSuccess)
        return err;
    const int64_t nrows = (int64_t)g.dims * g.dims;
    k_zifft_t1024<<<(unsigned)(nrows / kTRows), kTThreads, smem, stream>>>(
        reinterpret_cast<const float2 *>(kz_major), out, g.row, tw);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t kz_to_rows(const GridGeom &g, const float2 *kz_major, float2 *rows,
                       cudaStream_t stream, int64_t *launches)
{
    const dim3 grid((unsigned)((g.dims + 31) / 32), (unsigned)((g.hc + 31) / 32), (unsigned)g.dims);
    k_kz_to_rows<<<grid, 256, 0, stream>>>(kz_major, rows, g.dims, g.hc);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t yfft_pass(const GridGeom &g, float *grids, int nbatch, const float2 *tw, int num_sms,
                      cudaStream_t stream, int64_t *launches)
{
    const int n = g.dims;
    const int tz = xfft_tz(n);
    const int per_plane = (g.hc + tz - 1) / tz;
    const int64_t ntiles = (int64_t)per_plane * n * nbatch;
    const int ctas = (int)std::min<int64_t>(ntiles, (int64_t)num_sms * kXCtasPerSm);
    const size_t smem = 2 * kXTileBytes + sizeof(float2) * n;
    void (*kern)(float2 *, int, int, int64_t, const float2 *) = nullptr;
    switch (n) {
    case 64:
        kern = k_yfft<64>;
        break;
    case 128:
        kern = k_yfft<128>;
        break;
    case 256:
        kern = k_yfft<256>;
        break;
    case 512:
        kern = k_yfft<512>;
        break;
    default:
        return cudaErrorNotSupported;
    }
    cudaError_t err;
    if ((err = ensure_dynamic_smem(kern, smem)) != cudaSuccess)
        return err;
    kern<<<ctas, kXThreads, smem, stream>>>(reinterpret_cast<float2 *>(grids), g.hc, per_plane,
                                            ntiles, tw);
    (*launches)++;
    return cudaGetLastError();
}

int xfft_bin_ctas(int dims, int nbatch, int num_sms)
{
    const int tz = xfft_tz(dims);
    const int tiles = (dims * (dims / 2 + 1) + tz - 1) / tz * nbatch;
    return std::min(tiles, num_sms * kXCtasPerSm);
}

}  // namespace genpk
