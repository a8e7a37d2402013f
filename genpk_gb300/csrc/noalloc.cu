// noalloc.cu -- genpk_power_noalloc: the fused deconvolution + log-k binning of
// spectrum.cu for callers that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc: code running under a memory allocator
// that owns the whole device (a framework's caching pool, an embedding
// application that hands out only its own buffers), or a hot loop whose
// latency budget has no room for an allocation and its implicit
// synchronisation.  genpk_power needs a context, which allocates grids, cuFFT
// plans and scratch.  This entry point bins a spectrum the caller already has
// on the GPU and writes to the caller's output buffer; the only scratch it
// uses -- the per-CTA partial histograms and the bin tables -- lives in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.
//
// Limits (GENPK_NOALLOC_MAX_* in genpk_gb300.h): dims <= 1024, nrbins <= 1024.
// Larger requests fail with GENPK_ERR_UNSUPPORTED.  All calls share the one
// array and keep its last contents, so calls that overlap on the GPU (two
// streams, two host threads) race and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/genpk_gb300.h"
#include "internal.h"

namespace genpk {
namespace {

constexpr int kMaxDims = GENPK_NOALLOC_MAX_DIMS;
constexpr int kMaxBins = GENPK_NOALLOC_MAX_NRBINS;
constexpr int kMaxCtas = 304;  // binning CTAs: 2 per SM on a 152-SM GB300

constexpr size_t align256(size_t v)
{
    return (v + 255) & ~(size_t)255;
}

// Layout of the device scratch (bytes).
constexpr size_t kThrOff = 0;                                               // u32 [nrbins+1]
constexpr size_t kIwOff = kThrOff + align256(sizeof(uint32_t) * (kMaxBins + 1));  // f32 [dims]
constexpr size_t kCountOff = kIwOff + align256(sizeof(float) * kMaxDims);   // f64 [nrbins]
constexpr size_t kPartOff = kCountOff + align256(sizeof(double) * kMaxBins);  // f64 partials
constexpr size_t kScratchBytes = kPartOff + sizeof(double) * (size_t)kMaxCtas * kMaxBins;

// Host copies of the bin tables for the last (dims, nrbins) seen; static
// storage, so building them allocates nothing either.
constexpr int64_t kMaxHalf = kMaxDims / 2;
uint32_t h_thr[kMaxBins + 1];
float h_iw[kMaxDims];
int64_t h_count[kMaxBins];
double h_count_d[kMaxBins];
double h_keffs[kMaxBins];
int32_t h_lut[3 * kMaxHalf * kMaxHalf + 1];
int64_t h_cnt2[2 * kMaxHalf * kMaxHalf + 1];
double h_binsperunit = 0.0;
int64_t h_dims = -1;
int h_nrbins = -1;

constexpr int kMaxDevices = 64;
unsigned char *d_scratch[kMaxDevices];  // device address of the array, per device
int64_t d_dims[kMaxDevices];            // tables currently held on each device
int d_nrbins[kMaxDevices];

std::mutex g_mu;  // guards the host-side state above (not the GPU array)

}  // namespace
}  // namespace genpk

// The scratch itself.  Host code must not use this name as a device address:
// its address on each device comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_genpk_noalloc_scratch[genpk::kScratchBytes];

using namespace genpk;

extern "C" int genpk_power_noalloc(const float *spectrum_a, const float *spectrum_b, int64_t dims,
                                   int nrbins, double mass_a, double mass_b, double *power,
                                   int *count, double *keffs, void *stream)
{
    if (!spectrum_a || !power || dims < 2 || nrbins < 1)
        return GENPK_ERR_INVALID;
    if (dims > kMaxDims || nrbins > kMaxBins)
        return GENPK_ERR_UNSUPPORTED;
    if (!spectrum_b)
        spectrum_b = spectrum_a;
    cudaStream_t st = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(g_mu);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return GENPK_ERR_CUDA;

    // Set-up, once per device, with that device current.
    if (!d_scratch[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_genpk_noalloc_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return GENPK_ERR_CUDA;
        }
        d_scratch[dev] = (unsigned char *)ptr;
        d_dims[dev] = -1;
        d_nrbins[dev] = -1;
    }
    unsigned char *scratch = d_scratch[dev];

    // Bin tables: rebuilt on the host only when (dims, nrbins) changes.
    if (h_dims != dims || h_nrbins != nrbins) {
        TableSpans o{h_thr, h_iw, h_count, h_keffs, h_lut, h_cnt2};
        const char *why = nullptr;
        h_dims = -1;
        if (!build_bin_tables_into(dims, nrbins, o, &h_binsperunit, &why))
            return GENPK_ERR_UNSUPPORTED;
        for (int b = 0; b < nrbins; b++)
            h_count_d[b] = (double)h_count[b];
        h_dims = dims;
        h_nrbins = nrbins;
    }
    if (d_dims[dev] != dims || d_nrbins[dev] != nrbins) {
        if (cudaMemcpyAsync(scratch + kThrOff, h_thr, sizeof(uint32_t) * (nrbins + 1),
                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(scratch + kIwOff, h_iw, sizeof(float) * dims, cudaMemcpyHostToDevice,
                            st) != cudaSuccess ||
            cudaMemcpyAsync(scratch + kCountOff, h_count_d, sizeof(double) * nrbins,
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            cudaGetLastError();
            return GENPK_ERR_CUDA;
        }
        d_dims[dev] = dims;
        d_nrbins[dev] = nrbins;
    }

    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GENPK_ERR_CUDA;
    const GridGeom g = make_grid_geom((int)dims);
    const bool cross = spectrum_b != spectrum_a;
    int warps = 0;
    size_t smem = 0;
    int ctas = bin_ctas(g, nrbins, 1, cross ? 2 : 1, sms, &warps, &smem);
    if (ctas <= 0)
        return GENPK_ERR_UNSUPPORTED;
    ctas = ctas < kMaxCtas ? ctas : kMaxCtas;

    BinTables t;  // only the scalars are used by bin_spectra; no vectors are filled
    t.dims = dims;
    t.nrbins = nrbins;
    t.binsperunit = h_binsperunit;
    BinDevice d;
    d.thr = (uint32_t *)(scratch + kThrOff);
    d.iw = (float *)(scratch + kIwOff);
    d.count = (double *)(scratch + kCountOff);
    BinLaunch l;
    l.fields[0] = (const float2 *)spectrum_a;
    l.fields[1] = (const float2 *)spectrum_b;
    l.corner[0] = l.corner[1] = nullptr;
    l.nfields = cross ? 2 : 1;
    l.pairs[0].a = 0;
    l.pairs[0].b = cross ? 1 : 0;
    l.pairs[0].mass_a = mass_a;
    l.pairs[0].mass_b = mass_b;
    l.npairs = 1;
    int64_t launches = 0;
    if (bin_spectra(g, t, d, l, (double *)(scratch + kPartOff), power, ctas, warps, smem, st,
                    &launches) != cudaSuccess) {
        cudaGetLastError();
        return GENPK_ERR_CUDA;
    }
    for (int b = 0; b < nrbins; b++) {
        if (count)
            count[b] = (int)h_count[b];
        if (keffs)
            keffs[b] = h_keffs[b];
    }
    return GENPK_OK;
}
