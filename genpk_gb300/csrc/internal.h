// internal.h -- declarations shared by the host orchestration (genpk.cpp), the
// bin tables (tables.cpp) and the CUDA kernels (*.cu).  Not part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace genpk {

// ---------------------------------------------------------------------------
// Grid layout: dims x dims x row floats, row = 2*(dims/2+1) (the in-place r2c
// layout of gen-pk.cpp:176), x slowest.
// ---------------------------------------------------------------------------
struct GridGeom {
    int dims;        // N
    int half;        // N/2
    int hc;          // complex values per row: N/2+1
    int row;         // floats per row: 2*hc
    int64_t plane;   // floats per x-plane: row*N
    int64_t nfloat;  // floats in the grid: plane*N
};

GridGeom make_grid_geom(int dims);

// Raise `func`'s dynamic shared-memory limit on the current device to at
// least `bytes` (never lower it).  The limit is per kernel and device for the
// whole process, so contexts used from several host threads would otherwise
// race: one lowering it between another's set and launch fails that launch.
// Serialised by a process-wide mutex.
cudaError_t ensure_dynamic_smem(const void *func, size_t bytes);
template <typename F>
inline cudaError_t ensure_dynamic_smem(F *func, size_t bytes)
{
    return ensure_dynamic_smem(reinterpret_cast<const void *>(func), bytes);
}

// ---------------------------------------------------------------------------
// Deposit
// ---------------------------------------------------------------------------
struct DepositGeom {
    GridGeom grid;
    int tx, ty, tz;      // tile edge lengths in cells
    int ntx, nty, ntz;   // tiles per axis (ceil)
    int ntiles;
    int halo_per_tile;   // floats of halo scratch per tile
    float units_hi;      // dims/boxsize split into two floats (hi + lo)
    float units_lo;
};

// Scratch the deposit pass needs; owned by the context, grown on demand.
struct DepositScratch {
    uint32_t *hist = nullptr;        // [sort_ctas][ntiles]; becomes the scatter offsets
    size_t hist_cap = 0;             // elements
    uint32_t *tile_start = nullptr;  // [ntiles + 1]
    size_t tile_start_cap = 0;
    uint32_t *totals = nullptr;      // [ntiles]
    size_t tile_cap = 0;
    uint32_t *cursor = nullptr;      // [ntiles] scatter cursors (global-counter mode)
    size_t cursor_cap = 0;
    uint4 *sorted = nullptr;         // [cap] packed tile-local particles (x,y,z words, mass bits)
    size_t sorted_cap = 0;           // particles
    long long *faces = nullptr;      // [ntiles][face cells] 64-bit low-face sums
    size_t faces_cap = 0;
    long long *halo = nullptr;       // [ntiles][halo cells] 64-bit halo-layer sums
    size_t halo_cap = 0;
    double *mass_part = nullptr;     // [sort_ctas]
    int mass_part_cap = 0;
    unsigned long long *win_acc = nullptr;  // [nfloat] window engine's exact accumulator
};

// Device words a deposit pass reports through (zero-initialised).
struct DeviceStatus {
    unsigned long long bad_particles;  // non-finite positions/masses seen (skipped)
    unsigned long long timeouts;       // bounded waits that gave up
    double pass_mass;                  // mass deposited by the latest pass
    long long mean_fixed;              // pass mean in 2^-fx_shift mass units
    long long alt_sum;                 // sum over cells of (-1)^(x+y+z) * cell, fixed point
    int fx_shift;                      // weights are accumulated as round(w * 2^fx_shift)
    unsigned max_mass_bits;            // max |mass| of the pass, as float bits
};

struct DepositArgs {
    const float *pos;      // device [n][3]
    const float *masses;   // device [n] or nullptr
    float mass;            // uniform mass when masses == nullptr
    int64_t n;
    float *grid;           // device padded grid
    double *field_mass;    // device: running mass of this grid
    double *field_sub;     // device: running sum of the means subtracted from it
    double *field_corner;  // device: exact DFT value at k = (N/2, N/2, N/2), even N
    bool clean;            // grid content is undefined and must be overwritten
    bool host_mapped = false;  // pos/masses are pinned host memory read in place
    // Testing aid for the window engine's bounded waits (genpk_inject_copy_timeout):
    // chunk skip_chunk's bulk copy is not issued, and its wait gives up after
    // skip_wait clocks.  -1: none.
    int64_t skip_chunk = -1;
    long long skip_wait = 0;
};

// Tile shapes the deposit kernels are instantiated for.
struct TileShape {
    int tx, ty, tz;
};
bool deposit_tile_supported(int tx, int ty, int tz);
TileShape deposit_default_tile(int dims, int64_t n);
// Sort CTAs of a pass: up to max_per_sm per SM (fewer where the per-CTA tile
// histogram leaves no room), and no more than one per 4096 particles.
int deposit_sort_ctas(const DepositGeom &g, int64_t n, int num_sms, int max_per_sm = 1);
size_t deposit_hist_smem(const DepositGeom &g);
// True when the per-CTA tile histogram fits in shared memory (else the pass
// uses global counters).
bool deposit_shared_hist(const DepositGeom &g);
// 64-bit elements of face and halo scratch one pass needs.
void deposit_scratch_sizes(const DepositGeom &g, size_t *face_elems, size_t *halo_elems);

// Called after each kernel launch of a pass with the kernel's short name
// (used to record timing events); may be null.
typedef void (*StageHook)(void *user, const char *name);

// Launches the kernels of one deposit pass on `stream`.  Returns cudaSuccess
// or the first launch error.  *launches is incremented per kernel launched.
cudaError_t deposit_pass(const DepositGeom &g, const DepositArgs &a, DepositScratch &s,
                         DeviceStatus *dstat, int sort_ctas, cudaStream_t stream,
                         int64_t *launches, StageHook hook, void *hook_user);

// Grouped sorted-engine pass: the boxes of a batch that share a grid size go
// through one launch of each kernel of the pass.  Each box has its own
// particles, box size and mass, and its own clean grid (box b's at
// grid0 + b * grid_stride), field sums (field_mass0[b], field_sub0[b],
// field_corner0[b]) and status words (st0[b]).
constexpr int kMaxGroupBoxes = 32;
struct GroupBox {
    const float *pos;     // device [n][3]
    const float *masses;  // device [n] or nullptr
    float mass;           // uniform mass when masses == nullptr
    int64_t n;
    float units_hi, units_lo;  // dims/boxsize split into two floats
};
// Sort CTAs [cta0[b], cta0[b+1]) read box b's particles; its packed records
// are [rec0[b], rec0[b+1]) of the pass's record array.
struct GroupLayout {
    int nbox;
    int cta0[kMaxGroupBoxes + 1];
    int64_t rec0[kMaxGroupBoxes + 1];
};
// The pass's sort CTAs (deposit_sort_ctas over all the boxes' particles)
// shared out in proportion to the boxes' particles: at least one for a box
// with particles, none for an empty box, at most one per 4096 particles.
GroupLayout deposit_group_layout(int nbox, const GroupBox *boxes, int sort_ctas);
// Scratch elements a grouped pass needs beyond deposit_scratch_sizes per box:
// hist cta0[nbox] x ntiles, tile_start nbox x (ntiles + 1), totals
// nbox x ntiles, sorted rec0[nbox], mass_part cta0[nbox].  Requires
// deposit_shared_hist(g), nbox <= kMaxGroupBoxes and rec0[nbox] < 2^32.
// bad_out (device-visible, one word per box, may be null) receives each box's
// count of skipped particles, and the status word is zeroed for the next pass.
cudaError_t deposit_group_pass(const DepositGeom &g, const GroupLayout &lay, const GroupBox *boxes,
                               float *grid0, int64_t grid_stride, double *field_mass0,
                               double *field_sub0, double *field_corner0, DepositScratch &s,
                               DeviceStatus *st0, unsigned long long *bad_out, cudaStream_t stream,
                               int64_t *launches);

// Window engine (deposit_window.cu) for spatially coherent particle order.
constexpr int kWindowChunks[4] = {4096, 2048, 1024, 512};  // chunk lengths tried, largest first
// Shared window capacity in cells for a chunk length.
int window_cap_cells(int chunk, bool variable_masses);
// Window volume (cells) of `samples` evenly spread chunks, written to vol_dev.
cudaError_t window_probe(const DepositGeom &g, const DepositArgs &a, int chunk,
                         long long *vol_dev, int samples, cudaStream_t stream, int64_t *launches);
// Chunk length of the stream mode (no window: the chunk buffers only): 8192
// particles for uniform-mass passes of at least four such chunks per SM (one
// barrier per chunk: 1.32 -> 1.29 ms at 512^3, two 96 KB buffers), else 4096
// (variable masses would need 256 KB; smaller passes keep more chunks per CTA
// to balance).
constexpr int kStreamChunk = 4096;
constexpr int kStreamChunkLarge = 8192;
inline int stream_chunk(int64_t n, bool variable_masses, int num_sms)
{
    return (!variable_masses && n >= (int64_t)kStreamChunkLarge * 4 * num_sms) ? kStreamChunkLarge
                                                                              : kStreamChunk;
}
// Stream-mode merge count (out_dev[0]) out of neighbour pairs (out_dev[1]) over
// `samples` runs of 256 consecutive particles (none when fewer than 256).
cudaError_t stream_probe(const DepositGeom &g, const DepositArgs &a,
                         unsigned long long *out_dev, int samples, cudaStream_t stream,
                         int64_t *launches);
// One window-engine pass; mass_part needs mass_ctas doubles (variable masses);
// acc (nfloat 64-bit integers) is the exact accumulator.  stream_mode: the
// stream mode (reductions straight to acc, neighbour-merged), no windows.
// defer_convert (clean grids only): acc is left holding the pass, for
// zfft_pass to read or window_convert to turn into the FP32 grid later (both
// use the pass's mean and scale in dstat: no other pass may run before).
// clear_bytes: how much of acc, from its start, the pass clears first (all
// of it, or 0 when acc is known to hold zeros: cleared by the last
// transform's binning pass; or the part that a float grid overwrote).
cudaError_t deposit_window_pass(const DepositGeom &g, const DepositArgs &a, int chunk,
                                bool stream_mode, double *mass_part, int mass_ctas,
                                unsigned long long *acc, size_t clear_bytes, bool defer_convert,
                                int num_sms,
                                DeviceStatus *dstat, cudaStream_t stream, int64_t *launches,
                                StageHook hook, void *hook_user);
// The accumulator of the last window pass minus its mean, rounded once to FP32,
// into `grid` (clean: stored, else added).
cudaError_t window_convert(const GridGeom &g, const unsigned long long *acc, float *grid,
                           bool clean, const DeviceStatus *dstat, int num_sms,
                           cudaStream_t stream, int64_t *launches);

// ---------------------------------------------------------------------------
// Binning (deconvolution + log-k shells)
// ---------------------------------------------------------------------------
struct BinTables {
    int64_t dims = 0;
    int nrbins = 0;
    double binsperunit = 0.0;
    int64_t kk2max = 0;
    std::vector<uint32_t> thr;    // [nrbins+1]: smallest |k|^2 whose bin is >= b
    std::vector<float> iw;        // [dims]: float onedinvwindow(KVAL(i), dims)
    std::vector<int64_t> count;   // [nrbins] weighted mode counts
    std::vector<double> keffs;    // [nrbins] mean |k| (already divided by count)
    std::vector<int32_t> lut;     // [kk2max+1] bin of |k|^2 (-1 for 0)
};

// Build all tables with the reference's expressions.  Returns false and sets
// *err on failure (non-monotone bins, bin index out of range).
bool build_bin_tables(int64_t dims, int nrbins, BinTables *t, std::string *err);

// The same tables written into caller storage (no allocation):
// thr[nrbins+1], iw[dims], count[nrbins], keffs[nrbins], lut[table_kk2max+1],
// cnt2[table_r2max+1] (work space).
struct TableSpans {
    uint32_t *thr;
    float *iw;
    int64_t *count;
    double *keffs;
    int32_t *lut;
    int64_t *cnt2;
};
int64_t table_kk2max(int64_t dims);
int64_t table_r2max(int64_t dims);
bool build_bin_tables_into(int64_t dims, int nrbins, const TableSpans &o, double *binsperunit,
                           const char **why);
double ref_onedinvwindow(int64_t k, int64_t n);
double ref_invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n);

// x-axis FFT pass with optional fused auto-spectrum binning (xfft.cu), after
// the grid's (z, y) transforms (the own z and y passes, or a batched 2-D cuFFT
// R2C over x-planes).
struct XfftBin {
    int nrbins;
    float bpu_half;         // 0.5 * binsperunit (first-guess bin)
    const uint32_t *thr;    // [nrbins+1]
    const float *iw;        // [dims]
    const double *corner;   // exact (N/2,N/2,N/2) value per binned field, or null
    double *partial;        // [ctas][fields][nrbins] FP64 partial sums
    int fields = 1;         // 1, or the batch: each field's auto spectrum
};
bool xfft_supported(int dims);
bool xfft_bin_supported(int dims, int nrbins);
void xfft_twiddles(int dims, std::vector<float> *out);  // 2*dims floats
int xfft_bin_ctas(int dims, int nbatch, int num_sms);
// The z and y transforms of every x-plane for xfft_supported sizes (xfft.cu):
// zfft_pass is the length-N r2c along z of one grid, read from the window
// engine's 64-bit accumulator (converted as its conversion pass does, with the
// pass's mean and scale in dstat) and written to `grid`; yfft_pass is the
// complex length-N pass along y.  Followed by xfft_pass they leave the 3-D r2c
// transform.  xfft_pass also stores zeros over `zero_bytes` (a multiple of 16)
// at `zero`, when not null, spread over its tiles: the accumulator's clear for
// the next deposit pass, in HBM bandwidth that the binning x pass leaves idle
// (1.08 GB at N = 512 added 0.08 ms to it, against 0.15 ms for a separate
// clear; the y pass slowed more for half of it).
cudaError_t zfft_pass(const GridGeom &g, float *grid, const unsigned long long *acc,
                      const float2 *tw, const DeviceStatus *dstat, int num_sms,
                      cudaStream_t stream, int64_t *launches);
cudaError_t yfft_pass(const GridGeom &g, float *grids, int nbatch, const float2 *tw, int num_sms,
                      cudaStream_t stream, int64_t *launches);
// The kz-major z pass (xfft.cu, N = 1024): the length-N r2c along z of one
// grid read from the window engine's accumulator (converted as its conversion
// pass does) and written kz-major, S[kz][x][y] (N/2+1 planes of N x N complex
// values in the grid's memory), for a batched 2-D C2C over the planes to
// finish.
bool zfft_kz_supported(int dims);
// kz-major spectrum -> the in-place r2c layout, out of place (`rows` holds
// N * N * (N/2+1) complex values and must not overlap kz_major).
cudaError_t kz_to_rows(const GridGeom &g, const float2 *kz_major, float2 *rows,
                       cudaStream_t stream, int64_t *launches);
cudaError_t zfft_kz_pass(const GridGeom &g, float *grid, const unsigned long long *acc, const float2 *tw,
                         const DeviceStatus *dstat, cudaStream_t stream, int64_t *launches);
cudaError_t xfft_pass(const GridGeom &g, float *grids, int nbatch, const float2 *tw,
                      const XfftBin *bin, void *zero, int64_t zero_bytes, int num_sms,
                      DeviceStatus *dstat, cudaStream_t stream, int64_t *launches);
// The adjoint's first inverse pass (xfft.cu), for xfft_supported sizes: every
// mode of the spectrum in `grid` is scaled by its bin's coefficient gcoef[b]
// times V_m (the adjoint mode gradient), and the inverse (e^{+ikx})
// transform along x follows in the same pass.  A batched 2-D C2R over the
// x-planes then completes the unnormalised 3-D C2R.
struct XfftGrad {
    int nrbins;
    float bpu_half;
    const uint32_t *thr;
    const float *iw;
    const float *gcoef;  // [nrbins] G_b = 2 dL/dP_b / (M^2 C_b)
};
bool xfft_grad_supported(int dims, int nrbins);  // its bin tables fit in shared memory
cudaError_t xfft_grad_pass(const GridGeom &g, float *grid, const float2 *tw, const XfftGrad &grad,
                           int num_sms, DeviceStatus *dstat, cudaStream_t stream,
                           int64_t *launches);

struct BinDevice {
    uint32_t *thr = nullptr;   // [nrbins+1]
    float *iw = nullptr;       // [dims]
    double *count = nullptr;   // [nrbins] as double (exact up to 2^53)
    double *keffs = nullptr;   // [nrbins]
};

// One spectrum pair: indexes into the `fields` array of the launch.
struct BinPair {
    int a, b;
    double mass_a, mass_b;
};

constexpr int kMaxBinFields = 4;
constexpr int kMaxBinPairs = 10;

struct BinLaunch {
    const float2 *fields[kMaxBinFields];  // half-complex spectra (in-place layout)
    // Exact value of the (N/2, N/2, N/2) mode per field (device double), or null
    // to use the transform's own value.
    const double *corner[kMaxBinFields];
    int nfields;
    BinPair pairs[kMaxBinPairs];
    int npairs;
};

// Pair sums per CTA partial for a request (the instantiation's pair count:
// every pair of the fields, or the single pair of one or two fields).
int bin_pair_slots(int nfields, int npairs);
int bin_ctas(const GridGeom &g, int nrbins, int npairs, int nfields, int num_sms, int *warps,
             size_t *smem);

// Runs the binning kernel and the finalize kernel; writes out_power[np][nrbins]
// (device memory, or mapped host memory the kernel writes in place).
// partial must hold ctas*npairs*nrbins doubles.
// power[b] = sum over the CTA partials / (ma * mb * count[b]) (count 0: 0).
// With st_out, the finalize kernel also copies the status words *st_in there.
cudaError_t finalize_power(const double *partial, int ctas, int nrbins, const double *count,
                           double ma, double mb, double *out, cudaStream_t stream,
                           int64_t *launches, const DeviceStatus *st_in = nullptr,
                           DeviceStatus *st_out = nullptr);
// The same for the auto spectra of nfields fields binned together (partial:
// [ctas][nfields][nrbins]): out[f][nrbins] normalised by mass[f]^2, in
// launches of up to kMaxBinPairs fields; the last copies the status words.
cudaError_t finalize_powers(const double *partial, int ctas, int nrbins, int nfields,
                            const double *count, const double *mass, double *out,
                            cudaStream_t stream, int64_t *launches, const DeviceStatus *st_in,
                            DeviceStatus *st_out);
// Binning of one kz-major spectrum S[kz][x][y] (after zfft_kz_pass and the
// batched 2-D C2C): the auto pair's partial sums, one FP64 histogram per CTA
// (partial: ctas * nrbins doubles), for finalize_power.  When `zero` is not
// null the pass also stores zeros over zero_bytes (a multiple of 16) there,
// spread over its half-rows: the accumulator's clear for the next deposit
// pass, in HBM bandwidth the binning leaves idle.
int bin_kz_ctas(const GridGeom &g, int nrbins, int num_sms, int *warps, size_t *smem);
cudaError_t bin_spectrum_kz(const GridGeom &g, const BinTables &t, const BinDevice &d,
                            const float2 *spec, const double *corner, double *partial, int ctas,
                            int warps, size_t smem, void *zero, int64_t zero_bytes,
                            cudaStream_t stream, int64_t *launches);
cudaError_t bin_spectra(const GridGeom &g, const BinTables &t, const BinDevice &d,
                        const BinLaunch &l, double *partial, double *out_power, int ctas,
                        int warps, size_t smem, cudaStream_t stream, int64_t *launches,
                        const DeviceStatus *st_in = nullptr, DeviceStatus *st_out = nullptr);

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
// Replace the spectrum F in `spec` (in place) by the c2r input H of the
// density gradient for the auto spectrum: H_m = G_b V_m (c_m / mult_m) F_m with
// gcoef_dev[b] = G_b = 2 g_b / (M^2 C_b) (device, nrbins floats).
cudaError_t adjoint_mode_gradient_coef(const GridGeom &g, const BinTables &t, const BinDevice &d,
                                       float2 *spec, const float *gcoef_dev, cudaStream_t stream,
                                       int64_t *launches);

// The same on a kz-major spectrum S[kz][x][y] (the N = 1024 transform).
cudaError_t adjoint_mode_gradient_kz(const GridGeom &g, const BinTables &t, const BinDevice &d,
                                     float2 *spec, const float *gcoef_dev, int num_sms,
                                     cudaStream_t stream, int64_t *launches);
// The adjoint's inverse z pass for N = 1024 (xfft.cu): from the kz-major array
// left by the mode gradient and an inverse batched 2-D C2C over the kz planes,
// the unnormalised C2R along z of every row, written to `out` in the padded
// row layout (out must not overlap kz_major).
cudaError_t zifft_kz_pass(const GridGeom &g, const float *kz_major, float *out, const float2 *tw,
                          cudaStream_t stream, int64_t *launches);

// CIC gather of the real gradient grid: grad_pos[n][3], grad_mass[n] (optional).
cudaError_t adjoint_gather(const GridGeom &g, float units_hi, float units_lo, const float *grid,
                           const float *pos, const float *masses, float mass, int64_t n,
                           float *grad_pos, float *grad_mass, float dl_dmass_norm,
                           cudaStream_t stream, int64_t *launches);

int device_sm_count();

}  // namespace genpk
