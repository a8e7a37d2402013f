// genpk.cpp -- the C ABI (include/genpk_gb300.h): context, grid state, staging
// of host particles, cuFFT plans and the orchestration of the kernels in
// deposit.cu, spectrum.cu and adjoint.cu.
//
// Grid life cycle (per field):
//   CLEAN     after create / genpk_zero: contents undefined; the next deposit
//             pass overwrites instead of adding (no memset needed).
//   DENSITY   holds the mean-subtracted CIC density (FP32, padded layout).
//   SPECTRUM  holds its r2c transform in place (after genpk_power*).
//   GRADIENT  holds dL/drho after genpk_adjoint; must be zeroed before reuse.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/genpk_gb300.h"
#include "internal.h"

using namespace genpk;

namespace {

enum FieldState { F_CLEAN = 0, F_DENSITY = 1, F_SPECTRUM = 2, F_GRADIENT = 3 };

constexpr int kMaxStages = 64;
// Below this many particles a pass always uses the sorted engine.
constexpr int64_t kWindowMinParticles = (int64_t)1 << 20;
constexpr int64_t kZeroCopyMinParticles = (int64_t)1 << 20;
constexpr double kWindowMaxCellsPerParticle = 64.0;
// Coherent passes whose consecutive particles mostly advance one z cell along
// one (x, y) cell column (a lattice at about one particle per cell) take the
// stream mode: its neighbour merge then halves the reductions, and windows
// would merge few adds.  Measured at 512^3 particles (Zel'dovich lattice):
// merge rate 0.93 on a 512^3 grid (stream 1.41 ms, window 1.75 ms); 0.65 on
// 384^3 / 512^3, 0.49 on 512^3 / 256^3 and 0.02 on 256^3 / 512^3, where the
// window mode is 2-17 % faster.
constexpr double kStreamMergeRate = 0.8;

struct Pending {
    bool active = false;
    int field = -1;
    double boxsize = 0.0;
    bool varmass = false;
    float mass = 0.f;
};

}  // namespace

struct genpk_ctx {
    int64_t dims = 0;
    int nrbins = 0;
    int nfields = 0;
    unsigned flags = 0;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    GridGeom gg{};

    float *grids = nullptr;  // nfields contiguous grids of gg.nfloat floats
    std::vector<int> state;
    // [3*nfields]: deposited mass, subtracted mean, exact (N/2,N/2,N/2) mode
    double *d_field_mass = nullptr;
    std::vector<bool> corner_valid;  // the corner value belongs to the grid's spectrum
    DeviceStatus *d_status = nullptr;

    BinTables tables;
    BinDevice bdev;

    // cuFFT: r2c plans by batch size (3-D plans under +batch, batched 2-D
    // x-plane plans under -batch), one c2r plan; one shared work area.
    std::map<int, cufftHandle> r2c;
    int fft_mode = GENPK_FFT_AUTO;  // requested forward-FFT path
    float2 *d_xtw = nullptr;        // x-pass twiddles, null when unsupported
    cufftHandle c2r = 0;
    bool c2r_made = false;
    // N = 1024: batched 2-D C2C over the kz planes of a kz-major spectrum
    cufftHandle c2c_kz = 0;
    bool c2c_kz_made = false;
    // per field: its spectrum is kz-major, S[kz][x][y] (the N = 1024 transform)
    std::vector<bool> kzmajor;
    void *fft_work = nullptr;
    size_t fft_work_size = 0;

    // deposit
    TileShape tile{16, 16, 16};  // sorted engine's tile when fixed by the caller
    bool tile_fixed = false;     // genpk_set_deposit_tile chose it; else the tuner does
    // The sorted engine's tuned configurations, by particle-density band and
    // mass kind (chosen on the first clean pass of that band; see tune_sorted).
    struct Tuned {
        int band = 0;
        bool var = false;
        bool with_stream = false;         // the stream engine was among the trials
        int engine = GENPK_ENGINE_SORTED;  // the faster: SORTED (tile, per_sm) or STREAM
        TileShape tile{16, 16, 16};
        int per_sm = 1;
    };
    static constexpr int kTuned = 16;
    Tuned tuned[kTuned];
    int ntuned = 0;
    // the latest tuning's trials, and the configuration the latest sorted pass used
    static constexpr int kMaxTrials = 10;
    TileShape trial_tile[kMaxTrials];
    int trial_ctas[kMaxTrials] = {};
    float trial_ms[kMaxTrials] = {};
    int ntrials = 0;
    TileShape last_tile{16, 16, 16};
    int last_sort_ctas = 0;
    DepositScratch dscr;
    int engine = GENPK_ENGINE_AUTO;   // requested deposit engine
    int last_engine = GENPK_ENGINE_AUTO;  // engine the latest pass used
    long long *d_probe = nullptr;     // window-engine probe results
    // A field whose latest (clean) window-engine pass is still only in the
    // 64-bit accumulator: the forward transform reads it from there (the
    // conversion pass is skipped); anything else converts it first.
    int acc_pending = -1;
    // The accumulator holds zeros (the transform's x pass cleared it after its
    // contents were used), so the next window pass skips its clear;
    // acc_spent: its contents were used (converted or read by the z pass) and
    // the next own x pass may clear it.
    bool acc_zero = false;
    bool acc_spent = false;
    // With acc_zero false: 0 when any of the accumulator may be non-zero, else
    // the length of its non-zero prefix (a float grid written over a cleared
    // accumulator: the kz-major adjoint's dL/drho, or a row-major copy of a
    // kz-major spectrum), which is all that the next window pass clears.
    size_t acc_dirty_bytes = 0;
    // Recent automatic engine choices and the arrays they were made for (a few:
    // one per species of a multi-species loop).  Every engine yields the same
    // grid, so reusing a choice for the same particle arrays (a loop over the
    // same buffers, positions updated in place) can only change the speed; it
    // saves the probes and their host round trip.
    struct Choice {
        const float *pos = nullptr, *masses = nullptr;
        int64_t n = -1;
        double boxsize = 0.0;
        int engine = 0, chunk = 0;
    };
    static constexpr int kChoices = 32;  // species of a loop, or a batch of boxes per grid size
    Choice choices[kChoices];
    int choice_next = 0;
    size_t probe_cap = 0;
    // genpk_inject_copy_timeout: applied to the next window-engine pass only
    int64_t inject_chunk = -1;
    long long inject_clocks = 0;

    // staging of host particles
    float *stage_pos = nullptr;
    float *stage_mass = nullptr;
    int64_t stage_cap = 0;
    int64_t stage_n = 0;
    // Staged host particles merge into one pass up to this count (16 bytes each
    // on the device: 17 GB at 2^30, one pass for a whole 1024^3 snapshot; four
    // passes of 2^28 cost four accumulator clears and conversions and lost the
    // kz-major transform).  Where the device cannot hold that much, the staged
    // pass is deposited early instead (ensure_stage).
    int64_t stage_limit = (int64_t)1 << 30;
    Pending pend;

    // binning
    double *d_partial = nullptr;
    size_t partial_cap = 0;
    // The results: mapped pinned host memory that the finalize kernel writes in
    // place (the spectra, then a copy of the status words), so no copy back
    // follows the binning.  res_dev is its device address.
    double *res_host = nullptr;
    double *res_dev = nullptr;
    size_t res_cap = 0;  // doubles
    std::vector<std::vector<double>> auto_power;  // cached auto spectrum per field
    std::vector<double> auto_mass;
    std::vector<bool> auto_valid;

    // a power request issued without waiting (genpk_batch_power, genpk_power_step)
    struct Deferred {
        bool active = false;
        int np = 0;
        std::vector<int> pairs;
        std::vector<double> mass;
    } deferred;
    // inside genpk_batch_power: pinned host input is read in place without
    // waiting for the pass (the batch waits once for every box)
    bool batch_mode = false;

    // genpk_power_step: a CUDA graph of the whole step, captured on the second
    // of two identical calls and replayed while they stay identical
    struct StepGraph {
        bool on = true;
        bool failed = false;
        int attempts = 0;
        int repeats = 0;
        bool have_last = false;
        std::vector<unsigned char> last;  // the previous call's arguments, serialised
        cudaGraphExec_t exec = nullptr;
        uint64_t digest = 0;
        int64_t launches = 0;
        int64_t replays = 0;
        std::vector<int> pairs;
        std::vector<double> mass;
        int np = 0;
    } step;

    // adjoint scratch
    float *d_gcoef = nullptr;
    float *adj_buf = nullptr;  // device staging for host pos/masses/gradients
    size_t adj_cap = 0;        // floats

    // timing
    cudaEvent_t ev[kMaxStages + 1] = {};
    const char *stage_name[kMaxStages] = {};
    int nev = 0;
    int64_t launches = 0;

    std::string err;
};

namespace {

int fail(genpk_ctx *ctx, int code, const std::string &msg)
{
    if (ctx)
        ctx->err = msg;
    return code;
}

size_t acc_bytes(const genpk_ctx *ctx)
{
    return sizeof(unsigned long long) * (size_t)ctx->gg.nfloat;
}

// The accumulator's first `bytes` bytes were overwritten (used as a float
// buffer): only they need clearing if the rest was zero.
void acc_overwritten(genpk_ctx *ctx, size_t bytes)
{
    if (ctx->acc_zero)
        ctx->acc_dirty_bytes = bytes;
    else if (ctx->acc_dirty_bytes)
        ctx->acc_dirty_bytes = std::max(ctx->acc_dirty_bytes, bytes);
    ctx->acc_zero = false;
}

#define GENPK_CUDA(call)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? GENPK_ERR_NOMEM : GENPK_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

#define GENPK_CUFFT(call)                                                                     \
    do {                                                                                      \
        cufftResult r_ = (call);                                                              \
        if (r_ != CUFFT_SUCCESS)                                                              \
            return fail(ctx, GENPK_ERR_CUFFT,                                                 \
                        std::string(#call) + ": cufft error " + std::to_string((int)r_));    \
    } while (0)

#define GENPK_TRY(expr)                                                                       \
    do {                                                                                      \
        int s_ = (expr);                                                                      \
        if (s_ != GENPK_OK)                                                                   \
            return s_;                                                                        \
    } while (0)

bool is_device_ptr(const void *p)
{
    if (!p)
        return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device address of pinned (page-locked, mapped) host memory, or null for
// anything else.  Kernels may read such memory in place over the host link.
const float *mapped_host(const float *p)
{
    if (!p)
        return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer)
        return nullptr;
    return (const float *)a.devicePointer;
}

template <typename T>
int grow(genpk_ctx *ctx, T **ptr, size_t *cap, size_t need)
{
    if (*cap >= need)
        return GENPK_OK;
    if (*ptr) {
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaFree(*ptr);
        *ptr = nullptr;
        *cap = 0;
    }
    GENPK_CUDA(cudaMalloc((void **)ptr, sizeof(T) * need));
    *cap = need;
    return GENPK_OK;
}

// Room for `need` doubles of results in mapped pinned host memory.
int grow_res(genpk_ctx *ctx, size_t need)
{
    if (ctx->res_cap >= need)
        return GENPK_OK;
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->res_host);
    ctx->res_host = ctx->res_dev = nullptr;
    ctx->res_cap = 0;
    GENPK_CUDA(cudaHostAlloc((void **)&ctx->res_host, sizeof(double) * need, cudaHostAllocMapped));
    GENPK_CUDA(cudaHostGetDevicePointer((void **)&ctx->res_dev, ctx->res_host, 0));
    ctx->res_cap = need;
    return GENPK_OK;
}

float *grid_of(genpk_ctx *ctx, int f)
{
    return ctx->grids + (size_t)f * (size_t)ctx->gg.nfloat;
}

void stage_event(genpk_ctx *ctx, const char *name)
{
    if (!(ctx->flags & GENPK_FLAG_TIMING) || ctx->nev > kMaxStages)
        return;
    if (ctx->nev > 0)
        ctx->stage_name[ctx->nev - 1] = name;
    cudaEventRecord(ctx->ev[ctx->nev], ctx->stream);
    ctx->nev++;
}

// Record the start event of a timing window if none is open.  Windows are
// opened lazily by the first work-issuing call after genpk_timing_reset.
void timing_touch(genpk_ctx *ctx)
{
    if ((ctx->flags & GENPK_FLAG_TIMING) && ctx->nev == 0)
        stage_event(ctx, nullptr);
}

void deposit_hook(void *user, const char *name)
{
    stage_event(static_cast<genpk_ctx *>(user), name);
}

int check_field(genpk_ctx *ctx, int f)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    if (f < 0 || f >= ctx->nfields)
        return fail(ctx, GENPK_ERR_INVALID, "field index " + std::to_string(f) + " out of range");
    return GENPK_OK;
}

// Read back and clear the device's error counters.  Only the counters: the
// rest of the status (the latest pass's mean and scale) is still needed by a
// pass whose conversion is deferred to the transform.
// The error counters of a status copy already on the host; non-zero ones are
// cleared on the device and reported.
constexpr size_t kStatusDoubles = (sizeof(DeviceStatus) + sizeof(double) - 1) / sizeof(double);

int report_status(genpk_ctx *ctx, const DeviceStatus &st)
{
    if (st.bad_particles || st.timeouts) {
        static_assert(offsetof(DeviceStatus, timeouts) == sizeof(unsigned long long),
                      "the two counters lead DeviceStatus");
        GENPK_CUDA(cudaMemsetAsync(ctx->d_status, 0, 2 * sizeof(unsigned long long), ctx->stream));
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
        if (st.timeouts)
            return fail(ctx, GENPK_ERR_TIMEOUT,
                        std::to_string(st.timeouts) + " bounded device wait(s) gave up");
        return fail(ctx, GENPK_ERR_BAD_INPUT,
                    std::to_string(st.bad_particles) +
                        " particle(s) with non-finite or out-of-range position/mass were skipped");
    }
    return GENPK_OK;
}

int collect_status(genpk_ctx *ctx)
{
    DeviceStatus st;
    GENPK_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof st, cudaMemcpyDeviceToHost, ctx->stream));
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    return report_status(ctx, st);
}

DepositGeom deposit_geom(genpk_ctx *ctx, double boxsize, TileShape tile)
{
    DepositGeom g;
    g.grid = ctx->gg;
    g.tx = tile.tx;
    g.ty = tile.ty;
    g.tz = tile.tz;
    const int n = (int)ctx->dims;
    g.ntx = (n + g.tx - 1) / g.tx;
    g.nty = (n + g.ty - 1) / g.ty;
    g.ntz = (n + g.tz - 1) / g.tz;
    g.ntiles = g.ntx * g.nty * g.ntz;
    g.halo_per_tile = (g.ty + 1) * (g.tz + 1) + g.tx * (g.tz + 1) + g.tx * g.ty;
    const double units = (double)ctx->dims / boxsize;
    g.units_hi = (float)units;
    g.units_lo = (float)(units - (double)g.units_hi);
    return g;
}

DepositGeom deposit_geom(genpk_ctx *ctx, double boxsize)
{
    return deposit_geom(ctx, boxsize, ctx->tile);
}

int ensure_stage(genpk_ctx *ctx, int64_t need);

// Scratch of one sorted-engine pass of n particles with geometry g.
int grow_sorted_scratch(genpk_ctx *ctx, const DepositGeom &g, int64_t n, int sort_ctas)
{
    DepositScratch &s = ctx->dscr;
    if (deposit_shared_hist(g)) {
        GENPK_TRY(grow(ctx, &s.hist, &s.hist_cap, (size_t)sort_ctas * g.ntiles));
    } else {
        GENPK_TRY(grow(ctx, &s.cursor, &s.cursor_cap, (size_t)g.ntiles));
    }
    GENPK_TRY(grow(ctx, &s.tile_start, &s.tile_start_cap, (size_t)g.ntiles + 1));
    GENPK_TRY(grow(ctx, &s.totals, &s.tile_cap, (size_t)g.ntiles + 1));
    GENPK_TRY(grow(ctx, &s.sorted, &s.sorted_cap, (size_t)std::max<int64_t>(n, 1)));
    size_t nface = 0, nhalo = 0;
    deposit_scratch_sizes(g, &nface, &nhalo);
    GENPK_TRY(grow(ctx, &s.faces, &s.faces_cap, nface));
    GENPK_TRY(grow(ctx, &s.halo, &s.halo_cap, nhalo));
    size_t mp = (size_t)s.mass_part_cap;
    GENPK_TRY(grow(ctx, &s.mass_part, &mp, (size_t)sort_ctas));
    s.mass_part_cap = (int)mp;
    return GENPK_OK;
}

// Particle-density band of a pass: half octaves of particles per cell.
int density_band(const genpk_ctx *ctx, int64_t n)
{
    const double cells = (double)ctx->dims * (double)ctx->dims * (double)ctx->dims;
    return (int)std::floor(2.0 * std::log2(std::max((double)n, 1.0) / cells));
}

constexpr int64_t kTuneMinParticles = (int64_t)1 << 16;
// Timed runs per candidate (the fastest counts): single runs of a small pass
// varied by 10-20 %, enough to flip close choices from run to run.
constexpr int kTuneReps = 2;

// The deposit autotuner for particle orders without spatial coherence.  On
// the first clean pass of a density band (and mass kind) it runs the pass once
// per candidate -- the sorted engine with tiles 8^3, 16x16x8 and 16^3, each
// with up to 1, 2 and 4 sort CTAs per SM, and (with_stream) the stream
// engine, whose reductions go straight to the accumulator -- timed with CUDA
// events, and keeps the fastest.  (Measured on uniform random particles: the
// stream engine is 2-2.6x faster at 1e6 particles, where the sort's fixed
// costs dominate, about even at 3e7 on a 128^3 grid, and 1.75x slower at 3e7
// on a 256^3 grid, whose accumulator exceeds the L2.)  Every candidate writes
// the same grid (the sums are exact), so the trials only cost time: each
// overwrites the clean grid, and the field's running sums and the error
// counters are put back before the next.  The chosen candidate then runs as
// the real pass.
int tune_sorted(genpk_ctx *ctx, int f, double boxsize, const DepositArgs &a, bool with_stream,
                const genpk_ctx::Tuned **out)
{
    static const TileShape tiles[] = {{8, 8, 8}, {16, 16, 8}, {16, 16, 16}};
    // sort CTAs per SM: fewer CTAs give each (CTA, tile) run of the scatter
    // more particles, so its 16-byte records share sectors in the L2; more
    // shorten a CTA's range (two waves of 1024-thread CTAs)
    static const int pers[] = {1, 2};
    const size_t stash = 0;  // the error counters are kept in the probe buffer meanwhile
    GENPK_TRY(grow(ctx, &ctx->d_probe, &ctx->probe_cap, (size_t)4));
    GENPK_CUDA(cudaMemcpyAsync(ctx->d_probe + stash, ctx->d_status, 2 * sizeof(long long),
                               cudaMemcpyDeviceToDevice, ctx->stream));
    cudaEvent_t e0, e1;
    GENPK_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(ctx, GENPK_ERR_CUDA, "tune_sorted: cudaEventCreate failed");
    }
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } ev{e0, e1};
    auto reset_field = [&]() -> int {
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + f, 0, sizeof(double), ctx->stream));
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + ctx->nfields + f, 0, sizeof(double),
                                   ctx->stream));
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + 2 * ctx->nfields + f, 0, sizeof(double),
                                   ctx->stream));
        return GENPK_OK;
    };
    genpk_ctx::Tuned best;
    best.band = density_band(ctx, a.n);
    best.var = a.masses != nullptr;
    best.with_stream = with_stream;
    float best_ms = 1e30f;
    ctx->ntrials = 0;
    if (with_stream && !ctx->dscr.win_acc) {
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
        if (cudaMalloc(&ctx->dscr.win_acc,
                       sizeof(unsigned long long) * (size_t)ctx->gg.nfloat) != cudaSuccess) {
            cudaGetLastError();
            ctx->dscr.win_acc = nullptr;  // no room: the sorted engine only
        }
    }
    if (with_stream && ctx->dscr.win_acc) {
        const DepositGeom g = deposit_geom(ctx, boxsize);
        const int mass_ctas = ctx->num_sms * 4;
        size_t mp = (size_t)ctx->dscr.mass_part_cap;
        GENPK_TRY(grow(ctx, &ctx->dscr.mass_part, &mp, (size_t)mass_ctas));
        ctx->dscr.mass_part_cap = (int)mp;
        float ms = 1e30f;
        for (int rep = 0; rep < kTuneReps; rep++) {
            GENPK_TRY(reset_field());
            GENPK_CUDA(cudaEventRecord(e0, ctx->stream));
            GENPK_CUDA(deposit_window_pass(g, a,
                                           stream_chunk(a.n, a.masses != nullptr, ctx->num_sms),
                                           true, ctx->dscr.mass_part, mass_ctas,
                                           ctx->dscr.win_acc, acc_bytes(ctx), false, ctx->num_sms,
                                           ctx->d_status, ctx->stream, &ctx->launches, nullptr,
                                           nullptr));
            GENPK_CUDA(cudaEventRecord(e1, ctx->stream));
            GENPK_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            GENPK_CUDA(cudaEventElapsedTime(&t, e0, e1));
            ms = std::min(ms, t);
        }
        ctx->acc_zero = false;  // it holds the trial's sums
        ctx->acc_dirty_bytes = 0;
        ctx->acc_spent = true;
        ctx->trial_tile[0] = TileShape{0, 0, 0};
        ctx->trial_ctas[0] = 0;
        ctx->trial_ms[0] = ms;
        ctx->ntrials = 1;
        best_ms = ms;
        best.engine = GENPK_ENGINE_STREAM;
    }
    for (const TileShape &t : tiles) {
        if (!deposit_tile_supported(t.tx, t.ty, t.tz))
            continue;
        int last_ctas = -1;
        for (int per : pers) {
            const DepositGeom g = deposit_geom(ctx, boxsize, t);
            const int ctas = deposit_sort_ctas(g, a.n, ctx->num_sms, per);
            if (ctas == last_ctas)  // capped to the same count: nothing new to try
                continue;
            last_ctas = ctas;
            GENPK_TRY(grow_sorted_scratch(ctx, g, a.n, ctas));
            float ms = 1e30f;
            for (int rep = 0; rep < kTuneReps; rep++) {
                GENPK_TRY(reset_field());
                GENPK_CUDA(cudaEventRecord(e0, ctx->stream));
                GENPK_CUDA(deposit_pass(g, a, ctx->dscr, ctx->d_status, ctas, ctx->stream,
                                        &ctx->launches, nullptr, nullptr));
                GENPK_CUDA(cudaEventRecord(e1, ctx->stream));
                GENPK_CUDA(cudaEventSynchronize(e1));
                float t = 0.f;
                GENPK_CUDA(cudaEventElapsedTime(&t, e0, e1));
                ms = std::min(ms, t);
            }
            if (ctx->ntrials < genpk_ctx::kMaxTrials) {
                ctx->trial_tile[ctx->ntrials] = t;
                ctx->trial_ctas[ctx->ntrials] = ctas;
                ctx->trial_ms[ctx->ntrials] = ms;
                ctx->ntrials++;
            }
            if (ms < best_ms) {
                best_ms = ms;
                best.engine = GENPK_ENGINE_SORTED;
                best.tile = t;
                best.per_sm = per;
            }
        }
    }
    GENPK_TRY(reset_field());
    GENPK_CUDA(cudaMemcpyAsync(ctx->d_status, ctx->d_probe + stash, 2 * sizeof(long long),
                               cudaMemcpyDeviceToDevice, ctx->stream));
    genpk_ctx::Tuned &slot = ctx->tuned[ctx->ntuned % genpk_ctx::kTuned];
    ctx->ntuned++;
    slot = best;
    *out = &slot;
    return GENPK_OK;
}

const genpk_ctx::Tuned *find_tuned(const genpk_ctx *ctx, int64_t n, bool var, bool with_stream)
{
    const int band = density_band(ctx, n);
    const int have = std::min(ctx->ntuned, genpk_ctx::kTuned);
    for (int i = 0; i < have; i++)
        if (ctx->tuned[i].band == band && ctx->tuned[i].var == var &&
            ctx->tuned[i].with_stream == with_stream)
            return &ctx->tuned[i];
    return nullptr;
}

// One deposit pass from device particle arrays, or (host_mapped) from pinned
// host arrays read in place by the window engine.
int flush_acc(genpk_ctx *ctx);
bool use_xfft(const genpk_ctx *ctx);
bool use_kz(const genpk_ctx *ctx);

int run_deposit(genpk_ctx *ctx, int f, double boxsize, const float *pos, const float *masses,
                float mass, int64_t n, bool host_mapped = false)
{
    GENPK_TRY(flush_acc(ctx));  // this pass reuses the accumulator
    if (n > 0xffffffffLL - 1)
        return fail(ctx, GENPK_ERR_UNSUPPORTED, "more than 2^32-1 particles in one pass");
    const DepositGeom g = deposit_geom(ctx, boxsize);
    DepositScratch &s = ctx->dscr;
    DepositArgs a;
    a.pos = pos;
    a.masses = masses;
    a.mass = mass;
    a.n = n;
    a.grid = grid_of(ctx, f);
    a.field_mass = ctx->d_field_mass + f;
    a.field_sub = ctx->d_field_mass + ctx->nfields + f;
    a.field_corner = ctx->d_field_mass + 2 * ctx->nfields + f;
    a.clean = ctx->state[(size_t)f] == F_CLEAN;
    StageHook hook = (ctx->flags & GENPK_FLAG_TIMING) ? deposit_hook : nullptr;

    int engine = ctx->engine;
    int chunk = kWindowChunks[0];
    timing_touch(ctx);  // the probes belong to the pass
    // (never for the staging buffer: it holds a different caller array each time)
    const genpk_ctx::Choice *hit = nullptr;
    if (engine == GENPK_ENGINE_AUTO && pos != ctx->stage_pos)
        for (const auto &c : ctx->choices)
            if (c.pos == pos && c.masses == masses && c.n == n && c.boxsize == boxsize)
                hit = &c;
    const bool reuse = hit != nullptr;
    if (reuse) {
        engine = hit->engine;
        chunk = hit->chunk;
    } else if (engine == GENPK_ENGINE_WINDOW ||
               (engine == GENPK_ENGINE_AUTO && n >= kWindowMinParticles)) {
        // Spatially coherent order (most snapshot layouts) -> window engine
        // (or its stream mode where windows hold about one particle per cell);
        // anything else -> sorted engine.  Decided on a sample of chunks for
        // each chunk length: the largest length whose windows fit (a smaller
        // chunk leaves more shared memory to the window) and whose windows
        // stay small per particle (the flush visits every window cell).
        const int samples = 64, nq = (int)(sizeof(kWindowChunks) / sizeof(kWindowChunks[0]));
        GENPK_TRY(grow(ctx, &ctx->d_probe, &ctx->probe_cap, (size_t)samples * nq + 2));
        long long vol[4 * 64 + 2];
        bool stream_order = false;
        if (engine == GENPK_ENGINE_AUTO) {  // the stream probe first: it may settle it
            unsigned long long *merge_dev =
                reinterpret_cast<unsigned long long *>(ctx->d_probe + (size_t)samples * nq);
            GENPK_CUDA(stream_probe(g, a, merge_dev, samples, ctx->stream, &ctx->launches));
            GENPK_CUDA(cudaMemcpyAsync(vol, merge_dev, 2 * sizeof(long long),
                                       cudaMemcpyDeviceToHost, ctx->stream));
            GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
            stream_order = vol[1] > 0 && (double)vol[0] >= kStreamMergeRate * (double)vol[1];
        }
        int best = -1;
        if (!stream_order) {
            for (int q = 0; q < nq; q++)
                GENPK_CUDA(window_probe(g, a, kWindowChunks[q], ctx->d_probe + (size_t)q * samples,
                                        samples, ctx->stream, &ctx->launches));
            GENPK_CUDA(cudaMemcpyAsync(vol, ctx->d_probe, sizeof(long long) * samples * nq,
                                       cudaMemcpyDeviceToHost, ctx->stream));
            GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
            for (int q = 0; q < nq && best < 0; q++) {
                const int c = kWindowChunks[q];
                const int got = (int)std::min<int64_t>(samples, (n + c - 1) / c);
                const long long cap = window_cap_cells(c, masses != nullptr);
                int fit = 0;
                double cells = 0.0;
                for (int i = 0; i < got; i++) {
                    fit += vol[q * samples + i] <= (long long)(0.9 * cap) ? 1 : 0;
                    cells += (double)vol[q * samples + i];
                }
                if (got > 0 && fit * 10 >= got * 9 &&
                    cells / ((double)got * c) <= kWindowMaxCellsPerParticle)
                    best = q;
            }
        }
        if (engine == GENPK_ENGINE_AUTO)
            engine = stream_order ? GENPK_ENGINE_STREAM
                                  : (best >= 0 ? GENPK_ENGINE_WINDOW : GENPK_ENGINE_SORTED);
        if (best >= 0)
            chunk = kWindowChunks[best];
    }
    if (engine == GENPK_ENGINE_AUTO)  // too few particles to judge the order
        engine = GENPK_ENGINE_SORTED;
    // An automatic pass without spatial coherence: the tuner picks between the
    // sorted engine (and its tile) and the stream engine, per density band.
    const genpk_ctx::Tuned *tuned = nullptr;
    const bool auto_sorted = ctx->engine == GENPK_ENGINE_AUTO && engine == GENPK_ENGINE_SORTED &&
                             !ctx->tile_fixed && !host_mapped;
    if (auto_sorted || (engine == GENPK_ENGINE_SORTED && !ctx->tile_fixed && !host_mapped)) {
        tuned = find_tuned(ctx, n, masses != nullptr, auto_sorted);
        if (!tuned && a.clean && n >= kTuneMinParticles) {
            GENPK_TRY(tune_sorted(ctx, f, boxsize, a, auto_sorted, &tuned));
            stage_event(ctx, "tune");
        }
        if (tuned && tuned->engine == GENPK_ENGINE_STREAM)
            engine = GENPK_ENGINE_STREAM;
    }
    if (ctx->engine == GENPK_ENGINE_AUTO && !reuse) {
        if (pos != ctx->stage_pos) {
            genpk_ctx::Choice &c = ctx->choices[ctx->choice_next];
            ctx->choice_next = (ctx->choice_next + 1) % genpk_ctx::kChoices;
            c.pos = pos;
            c.masses = masses;
            c.n = n;
            c.boxsize = boxsize;
            c.engine = engine;
            c.chunk = chunk;
        }
        stage_event(ctx, "probe");
    }
    if ((engine == GENPK_ENGINE_WINDOW || engine == GENPK_ENGINE_STREAM) && !s.win_acc) {
        // The window engine's accumulator (8 bytes per grid element) is allocated on first
        // use; where it does not fit (the largest grids) an automatic pass takes the sorted
        // engine, which needs no grid-sized scratch.
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
        if (cudaMalloc(&s.win_acc, sizeof(unsigned long long) * (size_t)g.grid.nfloat) !=
            cudaSuccess) {
            cudaGetLastError();
            s.win_acc = nullptr;
            if (ctx->engine != GENPK_ENGINE_AUTO)
                return fail(ctx, GENPK_ERR_NOMEM,
                            "window engine: the 64-bit accumulator does not fit in device memory");
            engine = GENPK_ENGINE_SORTED;
        }
    }
    const bool chunked = engine == GENPK_ENGINE_WINDOW || engine == GENPK_ENGINE_STREAM;
    if (engine == GENPK_ENGINE_STREAM)
        chunk = stream_chunk(n, masses != nullptr, ctx->num_sms);
    if (chunked && ctx->inject_chunk >= 0) {
        a.skip_chunk = ctx->inject_chunk;
        a.skip_wait = ctx->inject_clocks;
        ctx->inject_chunk = -1;
    }
    if (host_mapped && !chunked) {
        // The sorted engine reads positions twice: copy them over once instead.
        GENPK_TRY(ensure_stage(ctx, n));
        GENPK_CUDA(cudaMemcpyAsync(ctx->stage_pos, pos, sizeof(float) * 3 * (size_t)n,
                                   cudaMemcpyDefault, ctx->stream));
        a.pos = ctx->stage_pos;
        if (masses) {
            GENPK_CUDA(cudaMemcpyAsync(ctx->stage_mass, masses, sizeof(float) * (size_t)n,
                                       cudaMemcpyDefault, ctx->stream));
            a.masses = ctx->stage_mass;
        }
        host_mapped = false;
    }
    a.host_mapped = host_mapped;
    ctx->last_engine = engine;
    timing_touch(ctx);
    if (chunked) {
        const int mass_ctas = ctx->num_sms * 4;
        size_t mp = (size_t)s.mass_part_cap;
        GENPK_TRY(grow(ctx, &s.mass_part, &mp, (size_t)mass_ctas));
        s.mass_part_cap = (int)mp;
        // A clean grid headed for the own z/y/x transform keeps the pass in the
        // accumulator: the z pass converts it on the fly.
        const bool defer = a.clean && (use_xfft(ctx) || use_kz(ctx));
        // (a pass that fails part-way must not leave the accumulator marked clear)
        const size_t clear = ctx->acc_zero ? 0 : ctx->acc_dirty_bytes ? ctx->acc_dirty_bytes
                                                                       : acc_bytes(ctx);
        ctx->acc_zero = false;
        ctx->acc_dirty_bytes = 0;
        GENPK_CUDA(deposit_window_pass(g, a, chunk, engine == GENPK_ENGINE_STREAM, s.mass_part,
                                       mass_ctas, s.win_acc, clear, defer, ctx->num_sms,
                                       ctx->d_status, ctx->stream, &ctx->launches, hook, ctx));
        ctx->acc_spent = !defer;  // converted in the pass
        if (defer)
            ctx->acc_pending = f;
    } else {
        TileShape tile = ctx->tile;
        int per_sm = 1;
        if (tuned) {
            tile = tuned->tile;
            per_sm = tuned->per_sm;
        }
        const DepositGeom gs = deposit_geom(ctx, boxsize, tile);
        const int sort_ctas = deposit_sort_ctas(gs, n, ctx->num_sms, per_sm);
        GENPK_TRY(grow_sorted_scratch(ctx, gs, n, sort_ctas));
        ctx->last_tile = tile;
        ctx->last_sort_ctas = sort_ctas;
        GENPK_CUDA(deposit_pass(gs, a, s, ctx->d_status, sort_ctas, ctx->stream, &ctx->launches,
                                hook, ctx));
    }
    ctx->state[(size_t)f] = F_DENSITY;
    ctx->auto_valid[(size_t)f] = false;
    return GENPK_OK;
}

// The pending accumulator (if any) into its FP32 grid.
int flush_acc(genpk_ctx *ctx)
{
    if (ctx->acc_pending < 0)
        return GENPK_OK;
    const int f = ctx->acc_pending;
    ctx->acc_pending = -1;
    ctx->acc_spent = true;
    GENPK_CUDA(window_convert(ctx->gg, ctx->dscr.win_acc, grid_of(ctx, f), true, ctx->d_status,
                              ctx->num_sms, ctx->stream, &ctx->launches));
    stage_event(ctx, "win_convert");
    return GENPK_OK;
}

// Staged host deposits of the pending pass, then the pending accumulator:
// afterwards every grid holds what its state says.
int flush_staged(genpk_ctx *ctx);

int flush_pending(genpk_ctx *ctx)
{
    GENPK_TRY(flush_staged(ctx));
    return flush_acc(ctx);
}

int flush_staged(genpk_ctx *ctx)
{
    if (!ctx->pend.active)
        return GENPK_OK;
    const Pending p = ctx->pend;
    const int64_t n = ctx->stage_n;
    ctx->pend.active = false;
    ctx->stage_n = 0;
    return run_deposit(ctx, p.field, p.boxsize, ctx->stage_pos, p.varmass ? ctx->stage_mass : nullptr,
                       p.mass, n);
}

// Room in the staging area for `need` particles (the staged ones included).
// The area grows by doubling up to stage_limit; where the device has no room
// for that, it grows to `need` exactly, and where it has no room for that
// either, the staged pass is deposited first and the area sized for the new
// chunk alone.
int ensure_stage(genpk_ctx *ctx, int64_t need)
{
    if (ctx->stage_cap >= need)
        return GENPK_OK;
    int64_t want = std::max<int64_t>(need, std::min<int64_t>(ctx->stage_limit, 2 * ctx->stage_cap));
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    float *np = nullptr, *nm = nullptr;
    for (;;) {
        if (cudaMalloc(&np, sizeof(float) * 3 * (size_t)want) == cudaSuccess &&
            cudaMalloc(&nm, sizeof(float) * (size_t)want) == cudaSuccess)
            break;
        cudaGetLastError();
        cudaFree(np);
        np = nullptr;
        if (want > need) {
            want = need;
        } else if (ctx->stage_n > 0) {
            need -= ctx->stage_n;
            GENPK_TRY(flush_staged(ctx));
            GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
            if (ctx->stage_cap >= need)
                return GENPK_OK;
            want = need;
        } else {
            return fail(ctx, GENPK_ERR_NOMEM, "staging allocation failed");
        }
    }
    if (ctx->stage_n > 0) {
        GENPK_CUDA(cudaMemcpyAsync(np, ctx->stage_pos, sizeof(float) * 3 * ctx->stage_n,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
        GENPK_CUDA(cudaMemcpyAsync(nm, ctx->stage_mass, sizeof(float) * ctx->stage_n,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    cudaFree(ctx->stage_pos);
    cudaFree(ctx->stage_mass);
    ctx->stage_pos = np;
    ctx->stage_mass = nm;
    ctx->stage_cap = want;
    return GENPK_OK;
}

// planes: a batched 2-D R2C over every x-plane of `batch` consecutive grids
// (the x-axis pass then runs in xfft.cu); else the full 3-D R2C.
// The common tail of a new cuFFT plan: failure reported (the plan destroyed),
// the context's stream set, and the one work area that every plan shares grown
// to the new plan's need (every existing plan then points at the new area).
int finish_plan(genpk_ctx *ctx, cufftHandle h, cufftResult made, size_t ws, const char *what)
{
    if (made != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(ctx, GENPK_ERR_CUFFT, std::string("cufftMakePlanMany64 (") + what +
                                              ") failed: " + std::to_string((int)made));
    }
    GENPK_CUFFT(cufftSetStream(h, ctx->stream));
    if (ws > ctx->fft_work_size) {
        GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->fft_work);
        ctx->fft_work = nullptr;
        GENPK_CUDA(cudaMalloc(&ctx->fft_work, ws));
        ctx->fft_work_size = ws;
        for (auto &kv : ctx->r2c)
            GENPK_CUFFT(cufftSetWorkArea(kv.second, ctx->fft_work));
        if (ctx->c2r_made)
            GENPK_CUFFT(cufftSetWorkArea(ctx->c2r, ctx->fft_work));
        if (ctx->c2c_kz_made)
            GENPK_CUFFT(cufftSetWorkArea(ctx->c2c_kz, ctx->fft_work));
    }
    GENPK_CUFFT(cufftSetWorkArea(h, ctx->fft_work));
    return GENPK_OK;
}

int make_r2c(genpk_ctx *ctx, int batch, bool planes, cufftHandle *out)
{
    const int key = planes ? -batch : batch;
    auto it = ctx->r2c.find(key);
    if (it != ctx->r2c.end()) {
        *out = it->second;
        return GENPK_OK;
    }
    const long long n = ctx->dims;
    cufftHandle h;
    GENPK_CUFFT(cufftCreate(&h));
    GENPK_CUFFT(cufftSetAutoAllocation(h, 0));
    size_t ws = 0;
    cufftResult r;
    if (planes) {
        long long dims2[2] = {n, n};
        long long inembed[2] = {n, (long long)ctx->gg.row};
        long long onembed[2] = {n, (long long)ctx->gg.hc};
        r = cufftMakePlanMany64(h, 2, dims2, inembed, 1, n * ctx->gg.row, onembed, 1,
                                n * ctx->gg.hc, CUFFT_R2C, (long long)batch * n, &ws);
    } else {
        long long dims3[3] = {n, n, n};
        long long inembed[3] = {n, n, (long long)ctx->gg.row};
        long long onembed[3] = {n, n, (long long)ctx->gg.hc};
        r = cufftMakePlanMany64(h, 3, dims3, inembed, 1, (long long)ctx->gg.nfloat, onembed, 1,
                                (long long)ctx->gg.nfloat / 2, CUFFT_R2C, batch, &ws);
    }
    GENPK_TRY(finish_plan(ctx, h, r, ws, "r2c"));
    ctx->r2c[key] = h;
    *out = h;
    return GENPK_OK;
}

// The batched 2-D C2R over the x-planes (y and z), in place, that completes
// the adjoint's inverse transform after its own x pass; kept in the plan map
// under key 0 (the R2C plans use +-batch).
int make_c2r_planes(genpk_ctx *ctx, cufftHandle *out)
{
    auto it = ctx->r2c.find(0);
    if (it != ctx->r2c.end()) {
        *out = it->second;
        return GENPK_OK;
    }
    const long long n = ctx->dims;
    long long dims2[2] = {n, n};
    long long inembed[2] = {n, (long long)ctx->gg.hc};
    long long onembed[2] = {n, (long long)ctx->gg.row};
    cufftHandle h;
    GENPK_CUFFT(cufftCreate(&h));
    GENPK_CUFFT(cufftSetAutoAllocation(h, 0));
    size_t ws = 0;
    cufftResult r = cufftMakePlanMany64(h, 2, dims2, inembed, 1, n * ctx->gg.hc, onembed, 1,
                                        n * ctx->gg.row, CUFFT_C2R, n, &ws);
    GENPK_TRY(finish_plan(ctx, h, r, ws, "c2r planes"));
    ctx->r2c[0] = h;
    *out = h;
    return GENPK_OK;
}

int make_c2r(genpk_ctx *ctx)
{
    if (ctx->c2r_made)
        return GENPK_OK;
    const long long n = ctx->dims;
    long long dims3[3] = {n, n, n};
    long long inembed[3] = {n, n, (long long)ctx->gg.hc};
    long long onembed[3] = {n, n, (long long)ctx->gg.row};
    cufftHandle h;
    GENPK_CUFFT(cufftCreate(&h));
    GENPK_CUFFT(cufftSetAutoAllocation(h, 0));
    size_t ws = 0;
    cufftResult r = cufftMakePlanMany64(h, 3, dims3, inembed, 1, (long long)ctx->gg.nfloat / 2,
                                        onembed, 1, (long long)ctx->gg.nfloat, CUFFT_C2R, 1, &ws);
    GENPK_TRY(finish_plan(ctx, h, r, ws, "c2r"));
    ctx->c2r = h;
    ctx->c2r_made = true;
    return GENPK_OK;
}

// The own x pass (and, for a field pending in the accumulator, the own z and y
// passes) replace cuFFT's x axis for the supported sizes.
bool use_xfft(const genpk_ctx *ctx)
{
    return ctx->fft_mode == GENPK_FFT_AUTO && ctx->d_xtw != nullptr &&
           xfft_supported((int)ctx->dims);
}

// N = 1024: a single field pending in the accumulator is transformed by the
// kz-major z pass (reads and clears the accumulator) and one batched 2-D C2C
// over the kz planes, and binned in kz-major order.
bool use_kz(const genpk_ctx *ctx)
{
    return ctx->fft_mode == GENPK_FFT_AUTO && ctx->d_xtw != nullptr &&
           zfft_kz_supported((int)ctx->dims);
}

// Batched forward 2-D C2C over the N/2+1 contiguous N x N planes of a
// kz-major spectrum, in place.
int make_c2c_kz(genpk_ctx *ctx)
{
    if (ctx->c2c_kz_made)
        return GENPK_OK;
    const long long n = ctx->dims;
    long long dims2[2] = {n, n};
    cufftHandle h;
    GENPK_CUFFT(cufftCreate(&h));
    GENPK_CUFFT(cufftSetAutoAllocation(h, 0));
    size_t ws = 0;
    cufftResult r = cufftMakePlanMany64(h, 2, dims2, dims2, 1, n * n, dims2, 1, n * n, CUFFT_C2C,
                                        (long long)ctx->gg.hc, &ws);
    GENPK_TRY(finish_plan(ctx, h, r, ws, "c2c kz planes"));
    ctx->c2c_kz = h;
    ctx->c2c_kz_made = true;
    return GENPK_OK;
}

// A kz-major spectrum back to the in-place r2c layout every other consumer
// reads (cross spectra with other fields, the adjoint).  Out of place through
// the window engine's accumulator, which then needs a clear before its next
// pass.
int ensure_row_major(genpk_ctx *ctx, int f)
{
    if (!ctx->kzmajor[(size_t)f])
        return GENPK_OK;
    float2 *tmp = reinterpret_cast<float2 *>(ctx->dscr.win_acc);
    if (!tmp)
        return fail(ctx, GENPK_ERR_STATE, "kz-major spectrum without its work buffer");
    GENPK_CUDA(kz_to_rows(ctx->gg, reinterpret_cast<const float2 *>(grid_of(ctx, f)), tmp,
                          ctx->stream, &ctx->launches));
    GENPK_CUDA(cudaMemcpyAsync(grid_of(ctx, f), tmp, sizeof(float) * (size_t)ctx->gg.nfloat,
                               cudaMemcpyDeviceToDevice, ctx->stream));
    acc_overwritten(ctx, sizeof(float) * (size_t)ctx->gg.nfloat);
    ctx->acc_spent = false;
    ctx->kzmajor[(size_t)f] = false;
    stage_event(ctx, "kz_to_rows");
    return GENPK_OK;
}

// fused: when not null and its field is transformed alone, the x-pass also
// bins that field's auto spectrum into fused->bin (fused->done := true); at
// N = 1024 (kz_ctas > 0) the field pending in the accumulator takes the
// kz-major transform and is binned in that order (fused->done := true).
struct FusedAuto {
    int field;  // the binned field (the first of bin.fields consecutive ones)
    XfftBin bin;
    bool done;
    int kz_ctas = 0, kz_warps = 0;
    size_t kz_smem = 0;
};

// Bring every field in `need` to SPECTRUM form: pending deposits first, then
// one batched r2c per run of consecutive field indices.
int to_spectrum(genpk_ctx *ctx, const std::vector<int> &need, FusedAuto *fused = nullptr)
{
    GENPK_TRY(flush_staged(ctx));
    std::vector<int> todo;
    for (int f : need) {
        const int st = ctx->state[(size_t)f];
        if (st == F_GRADIENT)
            return fail(ctx, GENPK_ERR_STATE,
                        "field " + std::to_string(f) + " holds an adjoint gradient; zero it first");
        if (st == F_CLEAN) {
            GENPK_CUDA(cudaMemsetAsync(grid_of(ctx, f), 0, sizeof(float) * ctx->gg.nfloat,
                                       ctx->stream));
            ctx->state[(size_t)f] = F_DENSITY;
        }
        if (ctx->state[(size_t)f] == F_DENSITY)
            todo.push_back(f);
    }
    std::sort(todo.begin(), todo.end());
    todo.erase(std::unique(todo.begin(), todo.end()), todo.end());
    if (fused && fused->kz_ctas > 0 && use_kz(ctx) && todo.size() == 1 &&
        todo[0] == fused->field && ctx->acc_pending == fused->field && ctx->dscr.win_acc) {
        const int f = fused->field;
        timing_touch(ctx);
        stage_event(ctx, "host");
        float *grid = grid_of(ctx, f);
        GENPK_CUDA(zfft_kz_pass(ctx->gg, grid, ctx->dscr.win_acc, ctx->d_xtw, ctx->d_status,
                                ctx->stream, &ctx->launches));
        ctx->acc_pending = -1;
        ctx->acc_spent = true;
        stage_event(ctx, "zfft_kz");
        GENPK_TRY(make_c2c_kz(ctx));
        GENPK_CUFFT(cufftExecC2C(ctx->c2c_kz, (cufftComplex *)grid, (cufftComplex *)grid,
                                 CUFFT_FORWARD));
        stage_event(ctx, "fft2d_kz");
        // the binning also clears the accumulator the z pass has read
        GENPK_CUDA(bin_spectrum_kz(ctx->gg, ctx->tables, ctx->bdev,
                                   reinterpret_cast<const float2 *>(grid), fused->bin.corner,
                                   fused->bin.partial, fused->kz_ctas, fused->kz_warps,
                                   fused->kz_smem, ctx->dscr.win_acc,
                                   (int64_t)sizeof(unsigned long long) * ctx->gg.nfloat,
                                   ctx->stream, &ctx->launches));
        ctx->acc_spent = false;
        ctx->acc_zero = true;
        stage_event(ctx, "bin_kz");
        ctx->state[(size_t)f] = F_SPECTRUM;
        ctx->corner_valid[(size_t)f] = true;
        ctx->kzmajor[(size_t)f] = true;
        fused->done = true;
        return GENPK_OK;
    }
    const bool planes = use_xfft(ctx);
    // A field whose pass is still in the accumulator is transformed on its own
    // by the own z pass (which reads the accumulator) and y pass; other runs of
    // consecutive fields take one batched 2-D cuFFT over their x-planes.  Both
    // then run the x pass.
    const int pend = planes ? ctx->acc_pending : -1;
    if (ctx->acc_pending >= 0 && (pend < 0 || std::find(todo.begin(), todo.end(), pend) == todo.end()))
        GENPK_TRY(flush_acc(ctx));
    timing_touch(ctx);
    stage_event(ctx, "host");
    size_t i = 0;
    while (i < todo.size()) {
        size_t j = i + 1;
        if (todo[i] != pend)
            while (j < todo.size() && todo[j] == todo[j - 1] + 1 && todo[j] != pend)
                j++;
        const int batch = (int)(j - i);
        float *base = grid_of(ctx, todo[i]);
        if (planes) {
            if (todo[i] == pend) {
                GENPK_CUDA(zfft_pass(ctx->gg, base, ctx->dscr.win_acc, ctx->d_xtw, ctx->d_status,
                                     ctx->num_sms, ctx->stream, &ctx->launches));
                ctx->acc_pending = -1;
                ctx->acc_spent = true;
                stage_event(ctx, "zfft");
                GENPK_CUDA(yfft_pass(ctx->gg, base, 1, ctx->d_xtw, ctx->num_sms, ctx->stream,
                                     &ctx->launches));
                stage_event(ctx, "yfft");
            } else {
                cufftHandle h;
                GENPK_TRY(make_r2c(ctx, batch, true, &h));
                GENPK_CUFFT(cufftExecR2C(h, (cufftReal *)base, (cufftComplex *)base));
                stage_event(ctx, "fft");
            }
            const bool bin = fused && batch == fused->bin.fields && todo[i] == fused->field;
            // The accumulator's clear, once its pass has been used, rides on a
            // binning x pass, whose bin walk leaves HBM bandwidth idle; the plain
            // x pass is faster and became HBM-bound with it (0.19 -> 0.36 ms at
            // N = 512, against 0.15 ms for the separate clear).
            const bool clear = bin && ctx->acc_spent && ctx->acc_pending < 0 && ctx->dscr.win_acc;
            GENPK_CUDA(xfft_pass(ctx->gg, base, batch, ctx->d_xtw, bin ? &fused->bin : nullptr,
                                 clear ? ctx->dscr.win_acc : nullptr, clear ? (int64_t)acc_bytes(ctx) : 0,
                                 ctx->num_sms, ctx->d_status, ctx->stream, &ctx->launches));
            if (clear) {
                ctx->acc_spent = false;
                ctx->acc_zero = true;
            }
            stage_event(ctx, bin ? "xfft_bin" : "xfft");
            if (bin)
                fused->done = true;
        } else {
            cufftHandle h;
            GENPK_TRY(make_r2c(ctx, batch, false, &h));
            GENPK_CUFFT(cufftExecR2C(h, (cufftReal *)base, (cufftComplex *)base));
            stage_event(ctx, "fft");
        }
        for (size_t k = i; k < j; k++) {
            ctx->state[(size_t)todo[k]] = F_SPECTRUM;
            ctx->corner_valid[(size_t)todo[k]] = true;
        }
        i = j;
    }
    return GENPK_OK;
}

// The host side of a finished power request: count, keffs, the cached auto
// spectra, the device status.
int finish_power(genpk_ctx *ctx, int np, const int *pairs, const double *pair_mass,
                 const double *power, int *count, double *keffs,
                 const DeviceStatus *host_status = nullptr)
{
    const int nrb = ctx->nrbins;
    for (int b = 0; b < nrb; b++) {
        if (count)
            count[b] = (int)ctx->tables.count[(size_t)b];
        if (keffs)
            keffs[b] = ctx->tables.keffs[(size_t)b];
    }
    for (int q = 0; q < np; q++) {
        if (pairs[2 * q] == pairs[2 * q + 1] && pair_mass[2 * q] == pair_mass[2 * q + 1]) {
            const int f = pairs[2 * q];
            ctx->auto_power[(size_t)f].assign(power + (size_t)q * nrb, power + (size_t)(q + 1) * nrb);
            ctx->auto_mass[(size_t)f] = pair_mass[2 * q];
            ctx->auto_valid[(size_t)f] = true;
        }
    }
    return host_status ? report_status(ctx, *host_status) : collect_status(ctx);
}

int power_collect(genpk_ctx *ctx, double *power, int *count, double *keffs);

// deferred: issue everything and return without waiting; power_collect
// finishes it (the results land in the context's mapped host buffer).
int power_impl(genpk_ctx *ctx, int np, const int *pairs, const double *pair_mass,
               double *power, int *count, double *keffs, bool deferred = false)
{
    if (np <= 0 || !pairs || !pair_mass || (!power && !deferred))
        return fail(ctx, GENPK_ERR_INVALID, "genpk_power_multi: bad pair arguments");
    std::vector<int> fields;
    for (int q = 0; q < 2 * np; q++) {
        GENPK_TRY(check_field(ctx, pairs[q]));
        fields.push_back(pairs[q]);
    }
    const int nrb = ctx->nrbins;
    GENPK_TRY(grow_res(ctx, (size_t)np * nrb + kStatusDoubles));
    DeviceStatus *st_out = reinterpret_cast<DeviceStatus *>(ctx->res_dev + (size_t)np * nrb);
    // Staged host chunks become their pass first, so that the choice of
    // transform below sees the field as the density it is.
    GENPK_TRY(flush_staged(ctx));
    // A single auto spectrum of a field still to be transformed: bin it inside
    // the x-axis FFT pass.
    FusedAuto fa;
    fa.done = false;
    FusedAuto *fused = nullptr;
    if (np == 1 && pairs[0] == pairs[1] && pair_mass[0] == pair_mass[1] && use_xfft(ctx) &&
        xfft_bin_supported(ctx->dims, nrb) && ctx->state[(size_t)pairs[0]] != F_SPECTRUM &&
        ctx->state[(size_t)pairs[0]] != F_GRADIENT) {
        const int ctas = xfft_bin_ctas(ctx->dims, 1, ctx->num_sms);
        GENPK_TRY(grow(ctx, &ctx->d_partial, &ctx->partial_cap, (size_t)ctas * nrb));
        fa.field = pairs[0];
        fa.bin.nrbins = nrb;
        fa.bin.bpu_half = (float)(0.5 * ctx->tables.binsperunit);
        fa.bin.thr = ctx->bdev.thr;
        fa.bin.iw = ctx->bdev.iw;
        fa.bin.corner = ctx->d_field_mass + 2 * ctx->nfields + pairs[0];
        fa.bin.partial = ctx->d_partial;
        fused = &fa;
    }
    // The auto spectra of consecutive fields still to be transformed in one
    // batch (a batch's grouped boxes): each binned inside the x pass, one
    // histogram per field.
    bool autos = np > 1 && use_xfft(ctx) && xfft_bin_supported(ctx->dims, nrb) &&
                 (ctx->acc_pending < pairs[0] || ctx->acc_pending >= pairs[0] + np);
    for (int q = 0; autos && q < np; q++)
        autos = pairs[2 * q] == pairs[0] + q && pairs[2 * q + 1] == pairs[2 * q] &&
                pair_mass[2 * q] == pair_mass[2 * q + 1] &&
                ctx->state[(size_t)pairs[2 * q]] == F_DENSITY;
    if (autos) {
        const int ctas = xfft_bin_ctas(ctx->dims, np, ctx->num_sms);
        GENPK_TRY(grow(ctx, &ctx->d_partial, &ctx->partial_cap, (size_t)ctas * np * nrb));
        fa.field = pairs[0];
        fa.bin.nrbins = nrb;
        fa.bin.bpu_half = (float)(0.5 * ctx->tables.binsperunit);
        fa.bin.thr = ctx->bdev.thr;
        fa.bin.iw = ctx->bdev.iw;
        fa.bin.corner = ctx->d_field_mass + 2 * ctx->nfields + pairs[0];
        fa.bin.partial = ctx->d_partial;
        fa.bin.fields = np;
        fused = &fa;
    }
    const bool auto1 = np == 1 && pairs[0] == pairs[1] && pair_mass[0] == pair_mass[1];
    if (!fused && auto1 && use_kz(ctx) && ctx->state[(size_t)pairs[0]] == F_DENSITY) {
        const int ctas = bin_kz_ctas(ctx->gg, nrb, ctx->num_sms, &fa.kz_warps, &fa.kz_smem);
        if (ctas > 0) {
            GENPK_TRY(grow(ctx, &ctx->d_partial, &ctx->partial_cap, (size_t)ctas * nrb));
            fa.field = pairs[0];
            fa.kz_ctas = ctas;
            fa.bin.corner = ctx->d_field_mass + 2 * ctx->nfields + pairs[0];
            fa.bin.partial = ctx->d_partial;
            fused = &fa;
        }
    }
    GENPK_TRY(to_spectrum(ctx, fields, fused));
    std::sort(fields.begin(), fields.end());
    fields.erase(std::unique(fields.begin(), fields.end()), fields.end());
    if (!fa.done && auto1 && ctx->kzmajor[(size_t)pairs[0]]) {
        // re-binning a kz-major spectrum: the same kernel as its transform's
        int warps = 0;
        size_t smem = 0;
        const int ctas = bin_kz_ctas(ctx->gg, nrb, ctx->num_sms, &warps, &smem);
        if (ctas > 0) {
            GENPK_TRY(grow(ctx, &ctx->d_partial, &ctx->partial_cap, (size_t)ctas * nrb));
            const int f = pairs[0];
            GENPK_CUDA(bin_spectrum_kz(
                ctx->gg, ctx->tables, ctx->bdev, reinterpret_cast<const float2 *>(grid_of(ctx, f)),
                ctx->corner_valid[(size_t)f] ? ctx->d_field_mass + 2 * ctx->nfields + f : nullptr,
                ctx->d_partial, ctas, warps, smem, nullptr, 0, ctx->stream, &ctx->launches));
            fa.kz_ctas = ctas;
            fa.done = true;
        }
    }
    if (!fa.done)  // every other binning reads the in-place r2c layout
        for (int f : fields)
            GENPK_TRY(ensure_row_major(ctx, f));
    if (fa.done && fa.bin.fields > 1) {
        std::vector<double> m((size_t)np);
        for (int q = 0; q < np; q++)
            m[(size_t)q] = pair_mass[2 * q];
        GENPK_CUDA(finalize_powers(ctx->d_partial, xfft_bin_ctas(ctx->dims, np, ctx->num_sms), nrb,
                                   np, ctx->bdev.count, m.data(), ctx->res_dev, ctx->stream,
                                   &ctx->launches, ctx->d_status, st_out));
    } else if (fa.done) {
        const int ctas =
            fa.kz_ctas > 0 ? fa.kz_ctas : xfft_bin_ctas(ctx->dims, 1, ctx->num_sms);
        GENPK_CUDA(finalize_power(ctx->d_partial, ctas, nrb, ctx->bdev.count, pair_mass[0],
                                  pair_mass[1], ctx->res_dev, ctx->stream, &ctx->launches,
                                  ctx->d_status, st_out));
    }
    // Pairs are binned in groups whose fields fit one kernel instantiation.
    int q0 = fa.done ? np : 0;
    while (q0 < np) {
        BinLaunch l;
        l.nfields = 0;
        l.npairs = 0;
        int q = q0;
        for (; q < np && l.npairs < kMaxBinPairs; q++) {
            int slot[2];
            int added = 0;
            for (int e = 0; e < 2; e++) {
                const float2 *fp = (const float2 *)grid_of(ctx, pairs[2 * q + e]);
                slot[e] = -1;
                for (int k = 0; k < l.nfields + added; k++)
                    if (l.fields[k] == fp)
                        slot[e] = k;
                if (slot[e] < 0) {
                    if (l.nfields + added >= kMaxBinFields) {
                        slot[e] = -2;
                    } else {
                        slot[e] = l.nfields + added;
                        l.fields[slot[e]] = fp;
                        const int fi = pairs[2 * q + e];
                        l.corner[slot[e]] = ctx->corner_valid[(size_t)fi]
                                                ? ctx->d_field_mass + 2 * ctx->nfields + fi
                                                : nullptr;
                        added++;
                    }
                }
            }
            if (slot[0] == -2 || slot[1] == -2)
                break;
            l.nfields += added;
            l.pairs[l.npairs].a = slot[0];
            l.pairs[l.npairs].b = slot[1];
            l.pairs[l.npairs].mass_a = pair_mass[2 * q];
            l.pairs[l.npairs].mass_b = pair_mass[2 * q + 1];
            l.npairs++;
        }
        int warps = 0;
        size_t smem = 0;
        const int ctas = bin_ctas(ctx->gg, nrb, l.npairs, l.nfields, ctx->num_sms, &warps, &smem);
        if (ctas <= 0)
            return fail(ctx, GENPK_ERR_UNSUPPORTED, "nrbins too large for the binning kernel");
        GENPK_TRY(grow(ctx, &ctx->d_partial, &ctx->partial_cap,
                       (size_t)ctas * bin_pair_slots(l.nfields, l.npairs) * nrb));
        const bool last = q >= np;  // the last finalize also copies the status words
        GENPK_CUDA(bin_spectra(ctx->gg, ctx->tables, ctx->bdev, l, ctx->d_partial,
                               ctx->res_dev + (size_t)q0 * nrb, ctas, warps, smem, ctx->stream,
                               &ctx->launches, ctx->d_status, last ? st_out : nullptr));
        q0 = q;
    }
    stage_event(ctx, "bin");
    ctx->deferred.active = true;
    ctx->deferred.np = np;
    ctx->deferred.pairs.assign(pairs, pairs + 2 * np);
    ctx->deferred.mass.assign(pair_mass, pair_mass + 2 * np);
    if (deferred)
        return GENPK_OK;
    return power_collect(ctx, power, count, keffs);
}

// Wait for a deferred power request and hand its results over.
int power_collect(genpk_ctx *ctx, double *power, int *count, double *keffs)
{
    if (!ctx->deferred.active)
        return fail(ctx, GENPK_ERR_STATE, "no power request is pending");
    ctx->deferred.active = false;
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    const genpk_ctx::Deferred &d = ctx->deferred;
    const size_t nv = (size_t)d.np * ctx->nrbins;
    memcpy(power, ctx->res_host, sizeof(double) * nv);
    DeviceStatus st;
    memcpy(&st, ctx->res_host + nv, sizeof st);
    return finish_power(ctx, d.np, d.pairs.data(), d.mass.data(), power, count, keffs, &st);
}

// A digest of everything in the context that decides which work a call
// issues, and where: state flags, cached choices, buffer addresses.  A batch
// replays a captured CUDA graph of a call only while every box's digest is
// the one it had when the call was captured.
uint64_t issue_digest(const genpk_ctx *ctx)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](uint64_t v) {
        for (int k = 0; k < 8; k++) {
            h ^= (v >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    };
    auto ptr = [&mix](const void *q) { mix((uint64_t)(uintptr_t)q); };
    for (int s : ctx->state)
        mix((uint64_t)s);
    for (bool v : ctx->corner_valid)
        mix(v);
    for (bool v : ctx->kzmajor)
        mix(v);
    mix((uint64_t)ctx->acc_pending);
    mix(ctx->acc_zero);
    mix(ctx->acc_spent);
    mix(ctx->acc_dirty_bytes);
    mix((uint64_t)ctx->engine);
    mix((uint64_t)ctx->last_engine);
    mix((uint64_t)ctx->fft_mode);
    mix((uint64_t)ctx->ntuned);
    mix((uint64_t)ctx->choice_next);
    mix(ctx->tile_fixed);
    mix((uint64_t)ctx->inject_chunk);
    mix(ctx->pend.active);
    mix((uint64_t)ctx->stage_n);
    mix(ctx->deferred.active);
    mix(ctx->c2r_made);
    mix(ctx->c2c_kz_made);
    mix(ctx->r2c.size());
    for (const void *q : {(const void *)ctx->grids, (const void *)ctx->d_field_mass,
                          (const void *)ctx->d_status, (const void *)ctx->d_xtw, (const void *)ctx->fft_work,
                          (const void *)ctx->dscr.hist, (const void *)ctx->dscr.tile_start,
                          (const void *)ctx->dscr.totals, (const void *)ctx->dscr.cursor,
                          (const void *)ctx->dscr.sorted, (const void *)ctx->dscr.faces,
                          (const void *)ctx->dscr.halo, (const void *)ctx->dscr.mass_part,
                          (const void *)ctx->dscr.win_acc, (const void *)ctx->d_probe,
                          (const void *)ctx->stage_pos, (const void *)ctx->stage_mass,
                          (const void *)ctx->d_partial, (const void *)ctx->res_dev})
        ptr(q);
    return h;
}

// The host-side record of what the device holds, which issuing a call
// updates as if its work had run.  A capture that fails runs nothing, so the
// record taken before it is put back.
struct IssueState {
    std::vector<int> state;
    std::vector<bool> corner_valid, kzmajor, auto_valid;
    std::vector<double> auto_mass;
    std::vector<std::vector<double>> auto_power;
    int acc_pending = -1;
    bool acc_zero = false, acc_spent = false;
    size_t acc_dirty_bytes = 0;
    int last_engine = 0;
    genpk_ctx::Deferred deferred;

    explicit IssueState(const genpk_ctx *c)
        : state(c->state), corner_valid(c->corner_valid), kzmajor(c->kzmajor),
          auto_valid(c->auto_valid), auto_mass(c->auto_mass), auto_power(c->auto_power),
          acc_pending(c->acc_pending), acc_zero(c->acc_zero), acc_spent(c->acc_spent),
          acc_dirty_bytes(c->acc_dirty_bytes), last_engine(c->last_engine), deferred(c->deferred)
    {
    }
    void restore(genpk_ctx *c) const
    {
        c->state = state;
        c->corner_valid = corner_valid;
        c->kzmajor = kzmajor;
        c->auto_valid = auto_valid;
        c->auto_mass = auto_mass;
        c->auto_power = auto_power;
        c->acc_pending = acc_pending;
        c->acc_zero = acc_zero;
        c->acc_spent = acc_spent;
        c->acc_dirty_bytes = acc_dirty_bytes;
        c->last_engine = last_engine;
        c->deferred = deferred;
    }
};

// Device copies of particle arrays for the adjoint when the caller passed host memory.
int adj_stage(genpk_ctx *ctx, size_t floats)
{
    return grow(ctx, &ctx->adj_buf, &ctx->adj_cap, floats);
}

int ctx_create(int64_t dims, int nrbins, int nfields, unsigned flags, genpk_ctx **out);

}  // namespace

extern "C" {

const char *genpk_status_string(int status)
{
    switch (status) {
    case GENPK_OK: return "ok";
    case GENPK_ERR_INVALID: return "invalid argument";
    case GENPK_ERR_CUDA: return "CUDA error";
    case GENPK_ERR_CUFFT: return "cuFFT error";
    case GENPK_ERR_NOMEM: return "out of memory";
    case GENPK_ERR_BAD_INPUT: return "bad particle data";
    case GENPK_ERR_STATE: return "invalid grid state";
    case GENPK_ERR_UNSUPPORTED: return "unsupported size or option";
    case GENPK_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char *genpk_last_error(const genpk_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : "null context";
}

void genpk_ctx_destroy(genpk_ctx *ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    if (ctx->step.exec)
        cudaGraphExecDestroy(ctx->step.exec);
    for (auto &kv : ctx->r2c)
        cufftDestroy(kv.second);
    if (ctx->c2r_made)
        cufftDestroy(ctx->c2r);
    if (ctx->c2c_kz_made)
        cufftDestroy(ctx->c2c_kz);
    cudaFree(ctx->fft_work);
    cudaFree(ctx->grids);
    cudaFree(ctx->d_field_mass);
    cudaFree(ctx->d_status);
    cudaFree(ctx->d_xtw);
    cudaFree(ctx->bdev.thr);
    cudaFree(ctx->bdev.iw);
    cudaFree(ctx->bdev.count);
    cudaFree(ctx->dscr.hist);
    cudaFree(ctx->dscr.tile_start);
    cudaFree(ctx->dscr.totals);
    cudaFree(ctx->dscr.sorted);
    cudaFree(ctx->dscr.halo);
    cudaFree(ctx->dscr.faces);
    cudaFree(ctx->dscr.cursor);
    cudaFree(ctx->dscr.mass_part);
    cudaFree(ctx->dscr.win_acc);
    cudaFree(ctx->stage_pos);
    cudaFree(ctx->stage_mass);
    cudaFree(ctx->d_partial);

    cudaFree(ctx->d_gcoef);
    cudaFree(ctx->adj_buf);
    cudaFree(ctx->d_probe);
    cudaFreeHost(ctx->res_host);
    for (auto &e : ctx->ev)
        if (e)
            cudaEventDestroy(e);
    if (ctx->stream)
        cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int genpk_ctx_create(int64_t dims, int nrbins, int nfields, unsigned flags, genpk_ctx **out)
{
    if (nfields > GENPK_MAX_FIELDS) {
        if (out)
            *out = nullptr;
        return GENPK_ERR_INVALID;
    }
    return ctx_create(dims, nrbins, nfields, flags, out);
}

}  // extern "C"

namespace {

// genpk_ctx_create without the public field limit: a batch's grouped boxes
// are the fields of one internal context (up to kMaxGroupBoxes).
int ctx_create(int64_t dims, int nrbins, int nfields, unsigned flags, genpk_ctx **out)
{
    if (!out)
        return GENPK_ERR_INVALID;
    *out = nullptr;
    if (dims < 2 || dims > 4096 || nrbins < 1 || nrbins > 65536 || nfields < 1 ||
        nfields > std::max(GENPK_MAX_FIELDS, kMaxGroupBoxes))
        return GENPK_ERR_INVALID;
    genpk_ctx *ctx = new genpk_ctx();
    ctx->dims = dims;
    ctx->nrbins = nrbins;
    ctx->nfields = nfields;
    ctx->flags = flags;
    ctx->gg = make_grid_geom((int)dims);
    int rc = GENPK_OK;
    auto bail = [&](int code) {
        *out = ctx;  // keep the error message readable; caller destroys
        return code;
    };
    std::string terr;
    if (!build_bin_tables(dims, nrbins, &ctx->tables, &terr)) {
        ctx->err = terr;
        return bail(GENPK_ERR_UNSUPPORTED);
    }
#define CREATE_CUDA(call)                                                                     \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                    \
            return bail(e_ == cudaErrorMemoryAllocation ? GENPK_ERR_NOMEM : GENPK_ERR_CUDA);  \
        }                                                                                     \
    } while (0)
    CREATE_CUDA(cudaGetDevice(&ctx->device));
    CREATE_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    CREATE_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    for (auto &e : ctx->ev)
        CREATE_CUDA(cudaEventCreate(&e));
    CREATE_CUDA(cudaMalloc(&ctx->grids, sizeof(float) * (size_t)ctx->gg.nfloat * nfields));
    CREATE_CUDA(cudaMalloc(&ctx->d_field_mass, sizeof(double) * 3 * nfields));
    CREATE_CUDA(cudaMemset(ctx->d_field_mass, 0, sizeof(double) * 3 * nfields));
    CREATE_CUDA(cudaMalloc(&ctx->d_status, sizeof(DeviceStatus)));
    CREATE_CUDA(cudaMemset(ctx->d_status, 0, sizeof(DeviceStatus)));
    CREATE_CUDA(cudaMalloc(&ctx->bdev.thr, sizeof(uint32_t) * (nrbins + 1)));
    CREATE_CUDA(cudaMemcpy(ctx->bdev.thr, ctx->tables.thr.data(), sizeof(uint32_t) * (nrbins + 1),
                           cudaMemcpyHostToDevice));
    CREATE_CUDA(cudaMalloc(&ctx->bdev.iw, sizeof(float) * dims));
    CREATE_CUDA(cudaMemcpy(ctx->bdev.iw, ctx->tables.iw.data(), sizeof(float) * dims,
                           cudaMemcpyHostToDevice));
    std::vector<double> cnt((size_t)nrbins);
    for (int b = 0; b < nrbins; b++)
        cnt[(size_t)b] = (double)ctx->tables.count[(size_t)b];
    CREATE_CUDA(cudaMalloc(&ctx->bdev.count, sizeof(double) * nrbins));
    CREATE_CUDA(cudaMemcpy(ctx->bdev.count, cnt.data(), sizeof(double) * nrbins,
                           cudaMemcpyHostToDevice));
    CREATE_CUDA(cudaMalloc(&ctx->d_gcoef, sizeof(float) * nrbins));
    if (xfft_supported((int)dims) || zfft_kz_supported((int)dims)) {
        std::vector<float> tw;
        xfft_twiddles((int)dims, &tw);
        CREATE_CUDA(cudaMalloc(&ctx->d_xtw, sizeof(float) * tw.size()));
        CREATE_CUDA(cudaMemcpy(ctx->d_xtw, tw.data(), sizeof(float) * tw.size(),
                               cudaMemcpyHostToDevice));
    }
#undef CREATE_CUDA
    ctx->state.assign((size_t)nfields, F_CLEAN);
    ctx->auto_power.assign((size_t)nfields, {});
    ctx->auto_mass.assign((size_t)nfields, 0.0);
    ctx->auto_valid.assign((size_t)nfields, false);
    ctx->corner_valid.assign((size_t)nfields, false);
    ctx->kzmajor.assign((size_t)nfields, false);
    ctx->tile = deposit_default_tile((int)dims, 0);
    (void)rc;
    *out = ctx;
    return GENPK_OK;
}

}  // namespace

extern "C" {

int genpk_zero(genpk_ctx *ctx, int field)
{
    GENPK_TRY(check_field(ctx, field));
    cudaSetDevice(ctx->device);
    if (ctx->pend.active && ctx->pend.field == field)
        GENPK_TRY(flush_staged(ctx));
    if (ctx->acc_pending == field) {
        ctx->acc_pending = -1;  // its accumulator is not needed any more
        ctx->acc_spent = true;
    }
    ctx->state[(size_t)field] = F_CLEAN;
    ctx->auto_valid[(size_t)field] = false;
    ctx->kzmajor[(size_t)field] = false;
    GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + field, 0, sizeof(double), ctx->stream));
    GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + ctx->nfields + field, 0, sizeof(double),
                               ctx->stream));
    GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + 2 * ctx->nfields + field, 0, sizeof(double),
                               ctx->stream));
    return GENPK_OK;
}

int genpk_deposit(genpk_ctx *ctx, int field, double boxsize, const float *pos, const float *masses,
                  double mass, int64_t n)
{
    GENPK_TRY(check_field(ctx, field));
    if (n < 0 || (n > 0 && !pos) || !(boxsize > 0.0) || !isfinite(boxsize))
        return fail(ctx, GENPK_ERR_INVALID, "genpk_deposit: bad n, pos or boxsize");
    if (!masses && !isfinite(mass))
        return fail(ctx, GENPK_ERR_INVALID, "genpk_deposit: non-finite uniform mass");
    cudaSetDevice(ctx->device);
    const int st = ctx->state[(size_t)field];
    if (st == F_SPECTRUM || st == F_GRADIENT)
        return fail(ctx, GENPK_ERR_STATE,
                    "field " + std::to_string(field) + " is not a density; call genpk_zero first");
    if (n == 0)
        return GENPK_OK;
    const bool pos_dev = is_device_ptr(pos);
    const bool mass_dev = masses ? is_device_ptr(masses) : pos_dev;
    if (pos_dev && mass_dev) {
        GENPK_TRY(flush_pending(ctx));
        return run_deposit(ctx, field, boxsize, pos, masses, (float)mass, n);
    }
    // Large pinned host arrays: the pass reads them in place, so the transfer
    // over the host link overlaps the deposit instead of preceding it.
    if (!pos_dev && n >= kZeroCopyMinParticles) {
        const float *pm = mapped_host(pos);
        const float *mm = masses ? (mass_dev ? masses : mapped_host(masses)) : nullptr;
        if (pm && (!masses || mm)) {
            GENPK_TRY(flush_pending(ctx));
            GENPK_TRY(run_deposit(ctx, field, boxsize, pm, mm, (float)mass, n, true));
            // The caller may free or reuse its buffers as soon as we return (a
            // batch waits for every box before it returns).
            if (!ctx->batch_mode)
                GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
            return GENPK_OK;
        }
    }
    // Stage host data on the device; merge with the pending pass when compatible.
    const bool var = masses != nullptr;
    const Pending &p = ctx->pend;
    const bool compatible = p.active && p.field == field && p.boxsize == boxsize &&
                            p.varmass == var && (var || p.mass == (float)mass);
    if (p.active && (!compatible || ctx->stage_n + n > ctx->stage_limit))
        GENPK_TRY(flush_pending(ctx));
    GENPK_TRY(ensure_stage(ctx, ctx->stage_n + n));
    const int64_t off = ctx->stage_n;
    GENPK_CUDA(cudaMemcpyAsync(ctx->stage_pos + 3 * off, pos, sizeof(float) * 3 * (size_t)n,
                               pos_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               ctx->stream));
    if (var)
        GENPK_CUDA(cudaMemcpyAsync(ctx->stage_mass + off, masses, sizeof(float) * (size_t)n,
                                   mass_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   ctx->stream));
    // The caller may free or reuse its host buffers as soon as we return.
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->stage_n += n;
    ctx->pend.active = true;
    ctx->pend.field = field;
    ctx->pend.boxsize = boxsize;
    ctx->pend.varmass = var;
    ctx->pend.mass = (float)mass;
    if (ctx->state[(size_t)field] == F_CLEAN)
        ctx->auto_valid[(size_t)field] = false;
    return GENPK_OK;
}

int genpk_power(genpk_ctx *ctx, int field_a, int field_b, double mass_a, double mass_b,
                double *power, int *count, double *keffs)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int pairs[2] = {field_a, field_b};
    const double masses[2] = {mass_a, mass_b};
    return power_impl(ctx, 1, pairs, masses, power, count, keffs);
}

int genpk_power_multi(genpk_ctx *ctx, int np, const int *pairs, const double *pair_mass,
                      double *power, int *count, double *keffs)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return power_impl(ctx, np, pairs, pair_mass, power, count, keffs);
}

int genpk_power_step(genpk_ctx *ctx, int nspecies, double boxsize, const float *const *pos,
                     const float *const *masses, const double *mass, const int64_t *n, int np,
                     const int *pairs, const double *pair_mass, double *power, int *count,
                     double *keffs)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    if (nspecies < 1 || nspecies > ctx->nfields || !pos || !mass || !n || np < 1 || !pairs ||
        !pair_mass || !power)
        return fail(ctx, GENPK_ERR_INVALID, "genpk_power_step: bad arguments");
    for (int q = 0; q < 2 * np; q++)
        if (pairs[q] < 0 || pairs[q] >= nspecies)
            return fail(ctx, GENPK_ERR_INVALID, "genpk_power_step: pair names a field past nspecies");
    cudaSetDevice(ctx->device);
    genpk_ctx::StepGraph &sg = ctx->step;
    if (ctx->deferred.active)
        return fail(ctx, GENPK_ERR_STATE, "genpk_power_step: a batch request is pending");

    std::vector<unsigned char> args;
    auto put = [&args](const void *v, size_t bytes) {
        const unsigned char *c = static_cast<const unsigned char *>(v);
        args.insert(args.end(), c, c + bytes);
    };
    put(&nspecies, sizeof nspecies);
    put(&boxsize, sizeof boxsize);
    put(pos, sizeof(*pos) * nspecies);
    for (int s = 0; s < nspecies; s++) {
        const float *m = masses ? masses[s] : nullptr;
        put(&m, sizeof m);
    }
    put(mass, sizeof(*mass) * nspecies);
    put(n, sizeof(*n) * nspecies);
    put(&np, sizeof np);
    put(pairs, sizeof(*pairs) * 2 * np);
    put(pair_mass, sizeof(*pair_mass) * 2 * np);
    if (sg.have_last && args == sg.last) {
        sg.repeats++;
    } else {
        if (sg.exec)
            cudaGraphExecDestroy(sg.exec);
        sg.exec = nullptr;
        sg.last = args;
        sg.have_last = true;
        sg.repeats = 0;
    }
    if (sg.exec && issue_digest(ctx) != sg.digest) {
        cudaGraphExecDestroy(sg.exec);  // the context was used otherwise since the capture
        sg.exec = nullptr;
    }

    auto issue = [&]() -> int {
        ctx->batch_mode = true;
        int rc = GENPK_OK;
        for (int s = 0; s < nspecies && rc == GENPK_OK; s++) {
            rc = genpk_zero(ctx, s);
            if (rc == GENPK_OK)
                rc = genpk_deposit(ctx, s, boxsize, pos[s], masses ? masses[s] : nullptr, mass[s],
                                   n[s]);
        }
        if (rc == GENPK_OK)
            rc = power_impl(ctx, np, pairs, pair_mass, nullptr, nullptr, nullptr, true);
        ctx->batch_mode = false;
        return rc;
    };

    // As for a batch: device-resident particles, no stage events.
    bool graphable = sg.on && !sg.failed && !(ctx->flags & GENPK_FLAG_TIMING);
    for (int s = 0; graphable && s < nspecies; s++)
        graphable = (n[s] == 0 || is_device_ptr(pos[s])) &&
                    (!masses || !masses[s] || is_device_ptr(masses[s]));
    if (graphable && !sg.exec && sg.repeats >= 1) {
        const uint64_t before = issue_digest(ctx);
        const IssueState saved(ctx);
        const int64_t launched = ctx->launches;
        bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        const bool began = ok;
        if (ok)
            ok = issue() == GENPK_OK;
        cudaGraph_t g = nullptr;
        if (began)
            ok = cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess && ok;
        const bool cuda_ok = ok;
        sg.launches = ctx->launches - launched;
        ctx->launches = launched;  // nothing ran yet
        sg.np = ctx->deferred.np;
        sg.pairs = ctx->deferred.pairs;
        sg.mass = ctx->deferred.mass;
        const bool pending = ctx->deferred.active;
        ctx->deferred.active = false;
        ok = ok && pending && issue_digest(ctx) == before;  // each replay starts where this did
        if (ok)
            ok = cudaGraphInstantiate(&sg.exec, g, 0) == cudaSuccess;
        if (g)
            cudaGraphDestroy(g);
        if (ok) {
            sg.digest = before;
            sg.attempts = 0;
        } else {
            cudaGetLastError();
            sg.exec = nullptr;
            if (!cuda_ok || ++sg.attempts >= 3)
                sg.failed = true;
            saved.restore(ctx);  // nothing ran
        }
    }
    if (sg.exec) {
        if (cudaGraphLaunch(sg.exec, ctx->stream) != cudaSuccess) {
            cudaGraphExecDestroy(sg.exec);
            sg.exec = nullptr;
            return fail(ctx, GENPK_ERR_CUDA, std::string("genpk_power_step: graph launch: ") +
                                                 cudaGetErrorString(cudaGetLastError()));
        }
        sg.replays++;
        ctx->launches += sg.launches;
        ctx->deferred.active = true;
        ctx->deferred.np = sg.np;
        ctx->deferred.pairs = sg.pairs;
        ctx->deferred.mass = sg.mass;
    } else {
        const int rc = issue();
        if (rc != GENPK_OK) {
            if (ctx->deferred.active)
                power_collect(ctx, power, count, keffs);
            return rc;
        }
    }
    return power_collect(ctx, power, count, keffs);
}

int genpk_power_step_use_graph(genpk_ctx *ctx, int on)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    genpk_ctx::StepGraph &sg = ctx->step;
    sg.on = on != 0;
    if (!sg.on && sg.exec) {
        cudaGraphExecDestroy(sg.exec);
        sg.exec = nullptr;
    }
    sg.failed = false;
    sg.attempts = 0;
    sg.repeats = 0;
    return GENPK_OK;
}

int64_t genpk_power_step_replays(const genpk_ctx *ctx)
{
    return ctx ? ctx->step.replays : -1;
}

double genpk_invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n)
{
    return ref_invwindow(kx, ky, kz, n);
}

int genpk_geometry(int64_t dims, int nrbins, int *count, double *keffs)
{
    if (dims < 2 || dims > 4096 || nrbins < 1 || !count || !keffs)
        return GENPK_ERR_INVALID;
    BinTables t;
    std::string err;
    if (!build_bin_tables(dims, nrbins, &t, &err))
        return GENPK_ERR_UNSUPPORTED;
    for (int b = 0; b < nrbins; b++) {
        count[b] = (int)t.count[(size_t)b];
        keffs[b] = t.keffs[(size_t)b];
    }
    return GENPK_OK;
}

int genpk_load_spectrum(genpk_ctx *ctx, int field, const double *spectrum)
{
    GENPK_TRY(check_field(ctx, field));
    if (!spectrum)
        return fail(ctx, GENPK_ERR_INVALID, "genpk_load_spectrum: null spectrum");
    cudaSetDevice(ctx->device);
    if (ctx->pend.active && ctx->pend.field == field)
        GENPK_TRY(flush_pending(ctx));
    const size_t nc = (size_t)ctx->gg.nfloat;  // 2 floats per complex value
    std::vector<float> tmp(nc);
    for (size_t i = 0; i < nc; i++)
        tmp[i] = (float)spectrum[i];
    GENPK_CUDA(cudaMemcpyAsync(grid_of(ctx, field), tmp.data(), sizeof(float) * nc,
                               cudaMemcpyHostToDevice, ctx->stream));
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->state[(size_t)field] = F_SPECTRUM;
    ctx->auto_valid[(size_t)field] = false;
    ctx->corner_valid[(size_t)field] = false;
    ctx->kzmajor[(size_t)field] = false;
    return GENPK_OK;
}

int genpk_bin_of(const genpk_ctx *ctx, int64_t kk2)
{
    if (!ctx || kk2 < 0 || kk2 > ctx->tables.kk2max)
        return -1;
    return ctx->tables.lut[(size_t)kk2];
}

int genpk_sync(genpk_ctx *ctx)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    cudaSetDevice(ctx->device);
    // A pass left in the accumulator counts as done: its grid is materialised
    // when something reads it.
    GENPK_TRY(flush_staged(ctx));
    return collect_status(ctx);
}

int genpk_read_field(genpk_ctx *ctx, int field, double *out)
{
    GENPK_TRY(check_field(ctx, field));
    if (!out)
        return fail(ctx, GENPK_ERR_INVALID, "genpk_read_field: null output");
    cudaSetDevice(ctx->device);
    GENPK_TRY(flush_pending(ctx));
    const int st = ctx->state[(size_t)field];
    const size_t nf = (size_t)ctx->gg.nfloat;
    if (st == F_CLEAN) {
        memset(out, 0, sizeof(double) * nf);
        return collect_status(ctx);
    }
    if (st != F_DENSITY)
        return fail(ctx, GENPK_ERR_STATE, "genpk_read_field: field is not a density");
    std::vector<float> tmp(nf);
    double mean = 0.0;  // the exact sum of the (fixed-point) means subtracted by the passes
    GENPK_CUDA(cudaMemcpyAsync(tmp.data(), grid_of(ctx, field), sizeof(float) * nf,
                               cudaMemcpyDeviceToHost, ctx->stream));
    GENPK_CUDA(cudaMemcpyAsync(&mean, ctx->d_field_mass + ctx->nfields + field, sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream));
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    const int row = ctx->gg.row, dims = (int)ctx->dims;
    for (size_t i = 0; i < nf; i++) {
        const int z = (int)(i % (size_t)row);
        out[i] = z < dims ? (double)tmp[i] + mean : 0.0;
    }
    return collect_status(ctx);
}

int genpk_adjoint(genpk_ctx *ctx, int field, double boxsize, const float *pos, const float *masses,
                  double mass, int64_t n, double mass_norm, const double *dl_dp, float *grad_pos,
                  float *grad_mass, double *dl_dmass_norm, int recompute)
{
    GENPK_TRY(check_field(ctx, field));
    if (n < 0 || (n > 0 && (!pos || !grad_pos)) || !dl_dp || !(boxsize > 0.0) ||
        !(mass_norm != 0.0) || (masses && !grad_mass))
        return fail(ctx, GENPK_ERR_INVALID, "genpk_adjoint: bad arguments");
    cudaSetDevice(ctx->device);
    GENPK_TRY(flush_pending(ctx));
    const bool dev = is_device_ptr(pos);
    if (dev != is_device_ptr(grad_pos) || (masses && dev != is_device_ptr(masses)) ||
        (grad_mass && dev != is_device_ptr(grad_mass)))
        return fail(ctx, GENPK_ERR_INVALID, "genpk_adjoint: mix of host and device pointers");
    const int nrb = ctx->nrbins;
    const float *dpos = pos, *dmass = masses;
    float *dgpos = grad_pos, *dgmass = grad_mass;
    if (!dev) {
        const size_t need = (size_t)n * (3 + 3) + (masses ? 2 * (size_t)n : 0) + 1;
        GENPK_TRY(adj_stage(ctx, need));
        float *b = ctx->adj_buf;
        float *sp = b, *sg = b + 3 * (size_t)n;
        float *sm = masses ? sg + 3 * (size_t)n : nullptr;
        float *sgm = masses ? sm + (size_t)n : nullptr;
        GENPK_CUDA(cudaMemcpyAsync(sp, pos, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice,
                                   ctx->stream));
        if (masses)
            GENPK_CUDA(cudaMemcpyAsync(sm, masses, sizeof(float) * (size_t)n,
                                       cudaMemcpyHostToDevice, ctx->stream));
        dpos = sp;
        dmass = sm;
        dgpos = sg;
        dgmass = sgm;
    }
    const bool have = ctx->state[(size_t)field] == F_SPECTRUM && ctx->auto_valid[(size_t)field] &&
                      ctx->auto_mass[(size_t)field] == mass_norm;
    std::vector<double> pw((size_t)nrb);
    if (recompute || !have) {
        ctx->state[(size_t)field] = F_CLEAN;
        ctx->kzmajor[(size_t)field] = false;
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + field, 0, sizeof(double), ctx->stream));
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + ctx->nfields + field, 0, sizeof(double),
                                   ctx->stream));
        GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass + 2 * ctx->nfields + field, 0,
                                   sizeof(double), ctx->stream));
        GENPK_TRY(run_deposit(ctx, field, boxsize, dpos, dmass, (float)mass, n));
        GENPK_TRY(genpk_power(ctx, field, field, mass_norm, mass_norm, pw.data(), nullptr, nullptr));
    } else {
        pw = ctx->auto_power[(size_t)field];
    }
    // A kz-major spectrum (N = 1024) takes the kz-major adjoint below.
    const bool kz = ctx->kzmajor[(size_t)field] && use_kz(ctx) && ctx->dscr.win_acc;
    if (!kz)
        GENPK_TRY(ensure_row_major(ctx, field));
    timing_touch(ctx);
    stage_event(ctx, "host");
    // dL/dM and the per-bin coefficients G_b = 2 g_b / (M^2 C_b).
    double dldm = 0.0;
    std::vector<float> gcoef((size_t)nrb, 0.f);
    for (int b = 0; b < nrb; b++) {
        dldm += dl_dp[b] * (-2.0 * pw[(size_t)b] / mass_norm);
        const double c = (double)ctx->tables.count[(size_t)b];
        if (c > 0)
            gcoef[(size_t)b] = (float)(2.0 * dl_dp[b] / (mass_norm * mass_norm * c));
    }
    if (dl_dmass_norm)
        *dl_dmass_norm = dldm;
    GENPK_CUDA(cudaMemcpyAsync(ctx->d_gcoef, gcoef.data(), sizeof(float) * nrb,
                               cudaMemcpyHostToDevice, ctx->stream));
    float *g = grid_of(ctx, field);
    if (kz) {
        // mode gradient in place, the inverse (x, y) transform per kz plane,
        // then the inverse z pass into the accumulator's memory (it cannot run
        // in place), which the gather reads; the accumulator needs a clear
        // before its next pass.
        GENPK_CUDA(adjoint_mode_gradient_kz(ctx->gg, ctx->tables, ctx->bdev, (float2 *)g,
                                            ctx->d_gcoef, ctx->num_sms, ctx->stream,
                                            &ctx->launches));
        stage_event(ctx, "adj_modes_kz");
        GENPK_TRY(make_c2c_kz(ctx));
        GENPK_CUFFT(cufftExecC2C(ctx->c2c_kz, (cufftComplex *)g, (cufftComplex *)g,
                                 CUFFT_INVERSE));
        stage_event(ctx, "adj_fft2d_kz");
        float *gbuf = reinterpret_cast<float *>(ctx->dscr.win_acc);
        GENPK_CUDA(zifft_kz_pass(ctx->gg, g, gbuf, ctx->d_xtw, ctx->stream, &ctx->launches));
        acc_overwritten(ctx, sizeof(float) * (size_t)ctx->gg.nfloat);
        ctx->acc_spent = false;
        ctx->kzmajor[(size_t)field] = false;
        g = gbuf;
        stage_event(ctx, "adj_c2r");
    } else if (use_xfft(ctx) && xfft_grad_supported((int)ctx->dims, nrb)) {
        // mode gradient fused into the inverse x pass, then the (y, z) C2R per x-plane
        XfftGrad xg;
        xg.nrbins = nrb;
        xg.bpu_half = (float)(0.5 * ctx->tables.binsperunit);
        xg.thr = ctx->bdev.thr;
        xg.iw = ctx->bdev.iw;
        xg.gcoef = ctx->d_gcoef;
        GENPK_CUDA(xfft_grad_pass(ctx->gg, g, ctx->d_xtw, xg, ctx->num_sms, ctx->d_status,
                                  ctx->stream, &ctx->launches));
        stage_event(ctx, "adj_modes_x");
        cufftHandle h;
        GENPK_TRY(make_c2r_planes(ctx, &h));
        GENPK_CUFFT(cufftExecC2R(h, (cufftComplex *)g, (cufftReal *)g));
    } else {
        GENPK_CUDA(adjoint_mode_gradient_coef(ctx->gg, ctx->tables, ctx->bdev, (float2 *)g,
                                              ctx->d_gcoef, ctx->stream, &ctx->launches));
        stage_event(ctx, "adj_modes");
        GENPK_TRY(make_c2r(ctx));
        GENPK_CUFFT(cufftExecC2R(ctx->c2r, (cufftComplex *)g, (cufftReal *)g));
    }
    ctx->state[(size_t)field] = F_GRADIENT;
    ctx->auto_valid[(size_t)field] = false;
    if (!kz)
        stage_event(ctx, "adj_c2r");
    const DepositGeom dg = deposit_geom(ctx, boxsize);
    GENPK_CUDA(adjoint_gather(ctx->gg, dg.units_hi, dg.units_lo, g, dpos, dmass, (float)mass, n,
                              dgpos, dgmass, (float)dldm, ctx->stream, &ctx->launches));
    stage_event(ctx, "adj_gather");
    if (!dev) {
        GENPK_CUDA(cudaMemcpyAsync(grad_pos, dgpos, sizeof(float) * 3 * (size_t)n,
                                   cudaMemcpyDeviceToHost, ctx->stream));
        if (masses)
            GENPK_CUDA(cudaMemcpyAsync(grad_mass, dgmass, sizeof(float) * (size_t)n,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    GENPK_CUDA(cudaStreamSynchronize(ctx->stream));
    return collect_status(ctx);
}

int genpk_timing_reset(genpk_ctx *ctx)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    ctx->nev = 0;
    return GENPK_OK;
}

int genpk_stage_times(const genpk_ctx *ctx, const char **names, float *ms, int cap)
{
    if (!ctx || !(ctx->flags & GENPK_FLAG_TIMING))
        return 0;
    int k = 0;
    for (int i = 0; i + 1 < ctx->nev && k < cap; i++, k++) {
        float t = 0.f;
        cudaEventSynchronize(ctx->ev[i + 1]);
        cudaEventElapsedTime(&t, ctx->ev[i], ctx->ev[i + 1]);
        if (names)
            names[k] = ctx->stage_name[i];
        if (ms)
            ms[k] = t;
    }
    return k;
}

int genpk_deposit_config(const genpk_ctx *ctx, int *tile_x, int *tile_y, int *tile_z,
                         int *sort_ctas)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    const bool ran = ctx->last_sort_ctas > 0;
    const TileShape t = ran ? ctx->last_tile : ctx->tile;
    if (tile_x)
        *tile_x = t.tx;
    if (tile_y)
        *tile_y = t.ty;
    if (tile_z)
        *tile_z = t.tz;
    if (sort_ctas) {
        if (ran) {
            *sort_ctas = ctx->last_sort_ctas;
        } else {
            DepositGeom g = deposit_geom(const_cast<genpk_ctx *>(ctx), 1.0);
            *sort_ctas = deposit_sort_ctas(g, (int64_t)1 << 30, ctx->num_sms);
        }
    }
    return GENPK_OK;
}

int genpk_deposit_trials(const genpk_ctx *ctx, int *tile_x, int *tile_y, int *tile_z,
                         int *sort_ctas, float *ms, int cap)
{
    if (!ctx || cap < 0)
        return -1;
    const int k = std::min(cap, ctx->ntrials);
    for (int i = 0; i < k; i++) {
        if (tile_x)
            tile_x[i] = ctx->trial_tile[i].tx;
        if (tile_y)
            tile_y[i] = ctx->trial_tile[i].ty;
        if (tile_z)
            tile_z[i] = ctx->trial_tile[i].tz;
        if (sort_ctas)
            sort_ctas[i] = ctx->trial_ctas[i];
        if (ms)
            ms[i] = ctx->trial_ms[i];
    }
    return k;
}

int genpk_set_deposit_tile(genpk_ctx *ctx, int tile_x, int tile_y, int tile_z)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    const bool automatic = tile_x == 0 && tile_y == 0 && tile_z == 0;
    if (!automatic && !deposit_tile_supported(tile_x, tile_y, tile_z))
        return fail(ctx, GENPK_ERR_UNSUPPORTED, "deposit tile shape not instantiated");
    GENPK_TRY(flush_pending(ctx));
    if (automatic) {
        ctx->tile_fixed = false;
        ctx->tile = deposit_default_tile((int)ctx->dims, 0);
    } else {
        ctx->tile_fixed = true;
        ctx->tile = TileShape{tile_x, tile_y, tile_z};
    }
    return GENPK_OK;
}

int genpk_set_deposit_engine(genpk_ctx *ctx, int engine)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    if (engine != GENPK_ENGINE_AUTO && engine != GENPK_ENGINE_SORTED &&
        engine != GENPK_ENGINE_WINDOW && engine != GENPK_ENGINE_STREAM)
        return fail(ctx, GENPK_ERR_INVALID, "unknown deposit engine");
    GENPK_TRY(flush_pending(ctx));
    ctx->engine = engine;
    return GENPK_OK;
}

int genpk_set_fft_mode(genpk_ctx *ctx, int mode)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    if (mode != GENPK_FFT_AUTO && mode != GENPK_FFT_CUFFT3D)
        return fail(ctx, GENPK_ERR_INVALID, "genpk_set_fft_mode: unknown mode");
    ctx->fft_mode = mode;
    return GENPK_OK;
}

int genpk_last_deposit_engine(const genpk_ctx *ctx)
{
    return ctx ? ctx->last_engine : -1;
}

int64_t genpk_kernel_launches(const genpk_ctx *ctx)
{
    return ctx ? ctx->launches : -1;
}

struct genpk_batch {
    std::vector<genpk_ctx *> box;
    std::vector<int64_t> dims;
    int nrbins = 0;
    unsigned flags = 0;
    std::string err;
    int mode = GENPK_BATCH_AUTO;
    int last_mode = -1;  // the way the latest call ran
    // GENPK_BATCH_AUTO: for calls of one shape (particle counts and mass
    // kinds), one untimed call each way (they tune), then one timed call each
    // way; later calls take the faster way.
    struct AutoChoice {
        std::vector<int64_t> key;
        int phase = 0;
        double ms[2] = {0.0, 0.0};
        int choice = GENPK_BATCH_PER_BOX;
    } au;

    // Grouped mode: the boxes of one grid size are the fields of one context
    // and share each kernel launch of a grouped sorted-engine pass.
    struct Group {
        genpk_ctx *ctx = nullptr;
        std::vector<int> boxes;                  // field f holds box boxes[f]
        DeviceStatus *d_st = nullptr;            // per box: the pass's status words
        unsigned long long *bad_host = nullptr;  // mapped: skipped particles per box
        unsigned long long *bad_dev = nullptr;
        bool tuned = false;
        std::vector<int64_t> tuned_n;  // the particle counts it was tuned for
        TileShape tile = {16, 16, 16};
        int per_sm = 1;
    };
    std::vector<Group> groups;

    // CUDA graph of a whole call.  A call with the same arguments as the one
    // before is captured (every unit's work -- a box, or a group of boxes --
    // forked from `origin` onto the units' streams and joined back) and later
    // identical calls replay it: one graph launch per call instead of one
    // launch per kernel.
    bool graph_on = true;
    bool graph_failed = false;  // a capture failed: calls stay eager
    int graph_attempts = 0;
    struct Args {
        std::vector<double> boxsize, mass, norm;
        std::vector<const float *> pos, masses;
        std::vector<int64_t> n;
        bool operator==(const Args &o) const
        {
            return boxsize == o.boxsize && mass == o.mass && norm == o.norm && pos == o.pos &&
                   masses == o.masses && n == o.n;
        }
    } last;
    bool have_last = false;
    int repeats = 0;  // consecutive calls with the arguments in `last`
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t exec = nullptr;
    bool graph_grouped = false;           // the graph is of a grouped call
    std::vector<int64_t> graph_launches;  // per unit: kernels one replay launches
    std::vector<genpk_ctx::Deferred> graph_deferred;
    std::vector<bool> graph_issued;
    std::vector<uint64_t> graph_digest;  // per unit, at capture
    int64_t replays = 0;
};

namespace {

void drop_graph(genpk_batch *b)
{
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

void destroy_groups(genpk_batch *b)
{
    for (genpk_batch::Group &g : b->groups) {
        genpk_ctx_destroy(g.ctx);
        cudaFree(g.d_st);
        cudaFreeHost(g.bad_host);
    }
    b->groups.clear();
}

// The groups of the grouped mode: boxes of one grid size, in the order of
// their first box, at most kMaxGroupBoxes to a group.
int make_groups(genpk_batch *b)
{
    if (!b->groups.empty())
        return GENPK_OK;
    const int nb = (int)b->box.size();
    std::vector<bool> taken((size_t)nb, false);
    for (int i = 0; i < nb; i++) {
        if (taken[(size_t)i])
            continue;
        genpk_batch::Group g;
        for (int j = i; j < nb && (int)g.boxes.size() < kMaxGroupBoxes; j++)
            if (!taken[(size_t)j] && b->dims[(size_t)j] == b->dims[(size_t)i]) {
                g.boxes.push_back(j);
                taken[(size_t)j] = true;
            }
        const int nf = (int)g.boxes.size();
        int rc = ctx_create(b->dims[(size_t)i], b->nrbins, nf, b->flags & ~GENPK_FLAG_TIMING,
                            &g.ctx);
        std::string why = rc != GENPK_OK && g.ctx ? genpk_last_error(g.ctx) : "";
        if (rc == GENPK_OK) {
            cudaError_t e = cudaMalloc(&g.d_st, sizeof(DeviceStatus) * (size_t)nf);
            if (e == cudaSuccess)
                e = cudaMemset(g.d_st, 0, sizeof(DeviceStatus) * (size_t)nf);
            if (e == cudaSuccess)
                e = cudaHostAlloc((void **)&g.bad_host, sizeof(unsigned long long) * (size_t)nf,
                                  cudaHostAllocMapped);
            if (e == cudaSuccess)
                e = cudaHostGetDevicePointer((void **)&g.bad_dev, g.bad_host, 0);
            if (e != cudaSuccess) {
                rc = e == cudaErrorMemoryAllocation ? GENPK_ERR_NOMEM : GENPK_ERR_CUDA;
                why = cudaGetErrorString(e);
                cudaGetLastError();
            }
        }
        b->groups.push_back(g);
        if (rc != GENPK_OK) {
            b->err = "group of box " + std::to_string(i) + ": " + why + " (" +
                     genpk_status_string(rc) + ")";
            destroy_groups(b);
            return rc;
        }
    }
    return GENPK_OK;
}

// Whether a call can run grouped: valid arguments (the per-box path reports
// the others, box by box), device-resident particles, grids whose tile
// histograms fit in shared memory, fewer than 2^32 particles per group.
bool groupable(const genpk_batch *b, const double *boxsize, const float *const *pos,
               const float *const *masses, const double *mass, const int64_t *n)
{
    const int nb = (int)b->box.size();
    for (int i = 0; i < nb; i++) {
        if (n[i] < 0 || (n[i] > 0 && !pos[i]) || !(boxsize[i] > 0.0) ||
            !std::isfinite(boxsize[i]) || (!(masses && masses[i]) && !std::isfinite(mass[i])))
            return false;
        if (n[i] > 0 && !is_device_ptr(pos[i]))
            return false;
        if (masses && masses[i] && n[i] > 0 && !is_device_ptr(masses[i]))
            return false;
        if (b->box[(size_t)i]->flags & GENPK_FLAG_TIMING)
            return false;
        DepositGeom g = deposit_geom(b->box[(size_t)i], 1.0, TileShape{16, 16, 16});
        if (!deposit_shared_hist(g))
            return false;
    }
    std::vector<int64_t> total;
    std::vector<int64_t> key;
    for (int i = 0; i < nb; i++) {
        size_t k = 0;
        while (k < key.size() && key[k] != b->dims[(size_t)i])
            k++;
        if (k == key.size()) {
            key.push_back(b->dims[(size_t)i]);
            total.push_back(0);
        }
        total[k] += n[i];
    }
    for (int64_t t : total)
        if (t > 0xfffffffeLL)
            return false;
    return true;
}

// Scratch of a grouped pass in the group context's sorted-engine buffers.
int grow_group_scratch(genpk_ctx *ctx, const DepositGeom &g, const GroupLayout &lay)
{
    DepositScratch &s = ctx->dscr;
    const int nb = lay.nbox;
    const int ctas = lay.cta0[nb];
    GENPK_TRY(grow(ctx, &s.hist, &s.hist_cap, std::max<size_t>(1, (size_t)ctas * g.ntiles)));
    GENPK_TRY(grow(ctx, &s.tile_start, &s.tile_start_cap, (size_t)nb * (g.ntiles + 1)));
    GENPK_TRY(grow(ctx, &s.totals, &s.tile_cap, (size_t)nb * g.ntiles + 1));
    GENPK_TRY(grow(ctx, &s.sorted, &s.sorted_cap, (size_t)std::max<int64_t>(lay.rec0[nb], 1)));
    size_t nface = 0, nhalo = 0;
    deposit_scratch_sizes(g, &nface, &nhalo);
    GENPK_TRY(grow(ctx, &s.faces, &s.faces_cap, nface * nb));
    GENPK_TRY(grow(ctx, &s.halo, &s.halo_cap, nhalo * nb));
    size_t mp = (size_t)s.mass_part_cap;
    GENPK_TRY(grow(ctx, &s.mass_part, &mp, (size_t)std::max(ctas, 1)));
    s.mass_part_cap = (int)mp;
    return GENPK_OK;
}

// One grouped pass of every box of group g into its field (which must be
// clean, with zero field sums).
int group_pass(genpk_batch::Group &g, const std::vector<GroupBox> &gb, TileShape tile, int per_sm)
{
    genpk_ctx *ctx = g.ctx;
    int64_t total = 0;
    for (const GroupBox &x : gb)
        total += x.n;
    const DepositGeom geo = deposit_geom(ctx, 1.0, tile);
    const int ctas = deposit_sort_ctas(geo, std::max<int64_t>(total, 1), ctx->num_sms, per_sm);
    const GroupLayout lay = deposit_group_layout((int)gb.size(), gb.data(), ctas);
    GENPK_TRY(grow_group_scratch(ctx, geo, lay));
    GENPK_CUDA(deposit_group_pass(geo, lay, gb.data(), ctx->grids, ctx->gg.nfloat, ctx->d_field_mass,
                                  ctx->d_field_mass + ctx->nfields, ctx->d_field_mass + 2 * ctx->nfields,
                                  ctx->dscr, g.d_st, g.bad_dev, ctx->stream, &ctx->launches));
    ctx->last_tile = tile;
    ctx->last_sort_ctas = lay.cta0[lay.nbox];
    ctx->last_engine = GENPK_ENGINE_SORTED;
    return GENPK_OK;
}

// The group's tile shape and sort CTAs per SM, timed as tune_sorted times
// the single-box candidates (the best of kTuneReps passes each); the trials
// are kept in the group context (genpk_deposit_trials).
int tune_group(genpk_batch::Group &g, const std::vector<GroupBox> &gb)
{
    static const TileShape tiles[] = {{8, 8, 8}, {16, 16, 8}, {16, 16, 16}};
    static const int pers[] = {1, 2};
    genpk_ctx *ctx = g.ctx;
    int64_t total = 0;
    for (const GroupBox &x : gb)
        total += x.n;
    cudaEvent_t e0, e1;
    GENPK_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(ctx, GENPK_ERR_CUDA, "tune_group: cudaEventCreate failed");
    }
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } ev{e0, e1};
    const size_t sums = sizeof(double) * 3 * (size_t)ctx->nfields;
    float best_ms = 1e30f;
    ctx->ntrials = 0;
    for (const TileShape &t : tiles) {
        const DepositGeom geo = deposit_geom(ctx, 1.0, t);
        if (!deposit_shared_hist(geo))
            continue;
        int last_ctas = -1;
        for (int per : pers) {
            const int ctas = deposit_sort_ctas(geo, std::max<int64_t>(total, 1), ctx->num_sms, per);
            if (ctas == last_ctas)
                continue;
            last_ctas = ctas;
            float ms = 1e30f;
            for (int rep = 0; rep < kTuneReps; rep++) {
                GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass, 0, sums, ctx->stream));
                GENPK_CUDA(cudaEventRecord(e0, ctx->stream));
                GENPK_TRY(group_pass(g, gb, t, per));
                GENPK_CUDA(cudaEventRecord(e1, ctx->stream));
                GENPK_CUDA(cudaEventSynchronize(e1));
                float x = 0.f;
                GENPK_CUDA(cudaEventElapsedTime(&x, e0, e1));
                ms = std::min(ms, x);
            }
            if (ctx->ntrials < genpk_ctx::kMaxTrials) {
                ctx->trial_tile[ctx->ntrials] = t;
                ctx->trial_ctas[ctx->ntrials] = ctas;
                ctx->trial_ms[ctx->ntrials] = ms;
                ctx->ntrials++;
            }
            if (ms < best_ms) {
                best_ms = ms;
                g.tile = t;
                g.per_sm = per;
            }
        }
    }
    GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass, 0, sums, ctx->stream));
    g.tuned = true;
    return GENPK_OK;
}

// Issues group g's work: every box deposited into its field by one grouped
// pass, then the auto spectra of all the fields (one batched transform of
// their x-planes, one x pass, binning of up to four fields per launch), to be
// collected by power_collect.
int group_issue(genpk_batch::Group &g, const double *boxsize, const float *const *pos,
                const float *const *masses, const double *mass, const int64_t *n,
                const double *mass_norm)
{
    genpk_ctx *ctx = g.ctx;
    const int nf = (int)g.boxes.size();
    cudaSetDevice(ctx->device);
    std::vector<GroupBox> gb((size_t)nf);
    std::vector<int64_t> counts((size_t)nf);
    for (int f = 0; f < nf; f++) {
        const int i = g.boxes[(size_t)f];
        const double units = (double)ctx->dims / boxsize[i];
        GroupBox &x = gb[(size_t)f];
        x.n = n[i];
        x.pos = n[i] > 0 ? pos[i] : nullptr;
        x.masses = masses && n[i] > 0 ? masses[i] : nullptr;
        x.mass = (float)mass[i];
        x.units_hi = (float)units;
        x.units_lo = (float)(units - (double)x.units_hi);
        counts[(size_t)f] = n[i];
        ctx->state[(size_t)f] = F_CLEAN;
        ctx->auto_valid[(size_t)f] = false;
        ctx->kzmajor[(size_t)f] = false;
        ctx->corner_valid[(size_t)f] = false;
    }
    GENPK_CUDA(cudaMemsetAsync(ctx->d_field_mass, 0, sizeof(double) * 3 * (size_t)ctx->nfields,
                               ctx->stream));
    if (!g.tuned || g.tuned_n != counts) {
        GENPK_TRY(tune_group(g, gb));
        g.tuned_n = counts;
    }
    GENPK_TRY(group_pass(g, gb, g.tile, g.per_sm));
    std::vector<int> pairs((size_t)2 * nf);
    std::vector<double> pm((size_t)2 * nf);
    for (int f = 0; f < nf; f++) {
        ctx->state[(size_t)f] = F_DENSITY;
        pairs[(size_t)2 * f] = pairs[(size_t)2 * f + 1] = f;
        pm[(size_t)2 * f] = pm[(size_t)2 * f + 1] = mass_norm[g.boxes[(size_t)f]];
    }
    return power_impl(ctx, nf, pairs.data(), pm.data(), nullptr, nullptr, nullptr, true);
}

}  // namespace

void genpk_batch_destroy(genpk_batch *b)
{
    if (!b)
        return;
    drop_graph(b);
    if (b->origin)
        cudaStreamDestroy(b->origin);
    if (b->fork)
        cudaEventDestroy(b->fork);
    for (cudaEvent_t e : b->join)
        cudaEventDestroy(e);
    for (genpk_ctx *c : b->box)
        genpk_ctx_destroy(c);
    destroy_groups(b);
    delete b;
}

int genpk_batch_use_graph(genpk_batch *b, int on)
{
    if (!b)
        return GENPK_ERR_INVALID;
    b->graph_on = on != 0;
    if (!b->graph_on)
        drop_graph(b);
    b->graph_failed = false;
    b->graph_attempts = 0;
    b->repeats = 0;
    return GENPK_OK;
}

int64_t genpk_batch_graph_replays(const genpk_batch *b)
{
    return b ? b->replays : -1;
}

int genpk_batch_set_mode(genpk_batch *b, int mode)
{
    if (!b || (mode != GENPK_BATCH_PER_BOX && mode != GENPK_BATCH_GROUPED &&
               mode != GENPK_BATCH_AUTO))
        return GENPK_ERR_INVALID;
    if (mode != b->mode) {
        drop_graph(b);
        b->repeats = 0;
        b->have_last = false;
        b->au = genpk_batch::AutoChoice{};
    }
    b->mode = mode;
    return GENPK_OK;
}

int genpk_batch_last_mode(const genpk_batch *b)
{
    return b ? b->last_mode : -1;
}

int genpk_batch_groups(const genpk_batch *b)
{
    return b ? (int)b->groups.size() : -1;
}

genpk_ctx *genpk_batch_group(genpk_batch *b, int g, int *nboxes, int *boxes)
{
    if (!b || g < 0 || g >= (int)b->groups.size())
        return nullptr;
    const genpk_batch::Group &gr = b->groups[(size_t)g];
    if (nboxes)
        *nboxes = (int)gr.boxes.size();
    if (boxes)
        for (size_t f = 0; f < gr.boxes.size(); f++)
            boxes[f] = gr.boxes[f];
    return gr.ctx;
}

int genpk_batch_create(int nboxes, const int64_t *dims, int nrbins, unsigned flags,
                       genpk_batch **out)
{
    if (!out)
        return GENPK_ERR_INVALID;
    *out = nullptr;
    if (nboxes < 1 || !dims || nrbins < 1)
        return GENPK_ERR_INVALID;
    genpk_batch *b = new genpk_batch();
    b->nrbins = nrbins;
    b->flags = flags;
    b->dims.assign(dims, dims + nboxes);
    for (int i = 0; i < nboxes; i++) {
        genpk_ctx *c = nullptr;
        const int rc = genpk_ctx_create(dims[i], nrbins, 1, flags, &c);
        if (rc != GENPK_OK) {
            b->err = "box " + std::to_string(i) + ": " + (c ? genpk_last_error(c) : "") +
                     " (" + genpk_status_string(rc) + ")";
            genpk_ctx_destroy(c);
            *out = b;  // keep the message readable; caller destroys
            return rc;
        }
        b->box.push_back(c);
    }
    *out = b;
    return GENPK_OK;
}

const char *genpk_batch_last_error(const genpk_batch *b)
{
    return b ? b->err.c_str() : "null batch";
}

genpk_ctx *genpk_batch_box(genpk_batch *b, int i)
{
    if (!b || i < 0 || i >= (int)b->box.size())
        return nullptr;
    return b->box[(size_t)i];
}

int64_t genpk_batch_launches(const genpk_batch *b)
{
    if (!b)
        return -1;
    int64_t k = 0;
    for (const genpk_ctx *c : b->box)
        k += c->launches;
    for (const genpk_batch::Group &g : b->groups)
        k += g.ctx->launches;
    return k;
}

int genpk_batch_power(genpk_batch *b, const double *boxsize, const float *const *pos,
                      const float *const *masses, const double *mass, const int64_t *n,
                      const double *mass_norm, double *power, int *count, double *keffs)
{
    if (!b)
        return GENPK_ERR_INVALID;
    const int nb = (int)b->box.size();
    if (!boxsize || !pos || !mass || !n || !mass_norm || !power) {
        b->err = "genpk_batch_power: null argument";
        return GENPK_ERR_INVALID;
    }
    const int nrb = b->nrbins;
    int first = GENPK_OK;
    auto note_msg = [&](int rc, const std::string &msg) {
        if (rc != GENPK_OK && first == GENPK_OK) {
            first = rc;
            b->err = msg;
        }
    };
    auto note = [&](int i, int rc) {
        if (rc != GENPK_OK)
            note_msg(rc, "box " + std::to_string(i) + ": " + genpk_last_error(b->box[(size_t)i]));
    };

    // The arguments, for the repeat test of the graph path.
    genpk_batch::Args args;
    args.boxsize.assign(boxsize, boxsize + nb);
    args.mass.assign(mass, mass + nb);
    args.norm.assign(mass_norm, mass_norm + nb);
    args.pos.assign(pos, pos + nb);
    args.masses.assign((size_t)nb, nullptr);
    if (masses)
        args.masses.assign(masses, masses + nb);
    args.n.assign(n, n + nb);
    const bool same = b->have_last && args == b->last;
    if (!same) {
        drop_graph(b);
        b->last = args;
        b->have_last = true;
        b->repeats = 0;
    } else {
        b->repeats++;
    }

    // Per box or grouped: as set, or (AUTO) by the trial calls' timings.
    const bool can_group = b->mode != GENPK_BATCH_PER_BOX &&
                           groupable(b, boxsize, pos, masses, mass, n);
    bool want_group = b->mode == GENPK_BATCH_GROUPED;
    bool trial = false;
    int timed_slot = -1;
    if (b->mode == GENPK_BATCH_AUTO && can_group) {
        genpk_batch::AutoChoice &au = b->au;
        std::vector<int64_t> key(n, n + nb);
        for (int i = 0; i < nb; i++)
            key.push_back(masses && masses[i] ? 1 : 0);
        if (key != au.key) {
            au = genpk_batch::AutoChoice{};
            au.key = key;
        }
        trial = au.phase < 4;
        want_group = trial ? (au.phase & 1) != 0 : au.choice == GENPK_BATCH_GROUPED;
        if (au.phase >= 2 && au.phase < 4)
            timed_slot = au.phase - 2;
    }
    const auto t_start = std::chrono::steady_clock::now();
    // The units of work: boxes (largest first, so that their passes start
    // first and the small ones fill in), or groups of boxes (largest first).
    bool grouped = want_group && can_group;
    const int made = grouped ? make_groups(b) : GENPK_OK;
    if (made != GENPK_OK) {
        // (the groups' contexts could not be made: the grouped mode reports
        // it; the automatic one runs per box from now on)
        if (b->mode == GENPK_BATCH_GROUPED)
            return made;
        b->mode = GENPK_BATCH_PER_BOX;
        b->err.clear();
        grouped = false;
        trial = false;
        timed_slot = -1;
    }
    std::vector<int> order;
    std::vector<genpk_ctx *> unit;
    if (grouped) {
        std::vector<int64_t> tot(b->groups.size(), 0);
        for (size_t g = 0; g < b->groups.size(); g++) {
            order.push_back((int)g);
            for (int i : b->groups[g].boxes)
                tot[g] += n[i];
        }
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return tot[(size_t)x] > tot[(size_t)y]; });
        for (const genpk_batch::Group &g : b->groups)
            unit.push_back(g.ctx);
    } else {
        for (int i = 0; i < nb; i++)
            order.push_back(i);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
        unit = b->box;
    }
    if (b->exec && b->graph_grouped != grouped)
        drop_graph(b);
    const int nu = (int)unit.size();
    std::vector<bool> issued((size_t)nu, false);
    auto issue = [&](int u) -> int {
        genpk_ctx *c = unit[(size_t)u];
        cudaSetDevice(c->device);
        int rc;
        if (grouped) {
            rc = group_issue(b->groups[(size_t)u], boxsize, pos, masses, mass, n, mass_norm);
        } else {
            c->batch_mode = true;
            rc = genpk_zero(c, 0);
            if (rc == GENPK_OK)
                rc = genpk_deposit(c, 0, boxsize[u], pos[u], masses ? masses[u] : nullptr,
                                   mass[u], n[u]);
            if (rc == GENPK_OK) {
                const int pr[2] = {0, 0};
                const double pm[2] = {mass_norm[u], mass_norm[u]};
                rc = power_impl(c, 1, pr, pm, nullptr, nullptr, nullptr, true);
            }
            c->batch_mode = false;
        }
        issued[(size_t)u] = rc == GENPK_OK;
        return rc;
    };
    bool group_nomem = false;  // a group's scratch did not fit
    auto note_unit = [&](int u, int rc) {
        if (rc == GENPK_OK)
            return;
        if (!grouped)
            return note(u, rc);
        group_nomem = group_nomem || rc == GENPK_ERR_NOMEM;
        note_msg(rc, "boxes of grid " + std::to_string(unit[(size_t)u]->dims) + ": " +
                         genpk_last_error(unit[(size_t)u]));
    };

    // One device, no stage events (a replay does not re-record them), and
    // particles in device memory: host input goes through host-side copies
    // into staging buffers, which a replay would not repeat.
    bool graphable = b->graph_on && !b->graph_failed && !trial;
    for (int i = 0; graphable && i < nb; i++) {
        const genpk_ctx *c = b->box[(size_t)i];
        graphable = c->device == b->box[0]->device && !(c->flags & GENPK_FLAG_TIMING) &&
                    (n[i] == 0 || is_device_ptr(pos[i])) &&
                    (!masses || !masses[i] || is_device_ptr(masses[i]));
    }
    if (b->exec) {
        for (int u = 0; u < nu; u++)
            if (issue_digest(unit[(size_t)u]) != b->graph_digest[(size_t)u] ||
                unit[(size_t)u]->deferred.active) {
                drop_graph(b);  // a unit was used on its own since the capture
                break;
            }
    }
    if (graphable && !b->exec && b->repeats >= 1) {
        // Capture this call: every unit's work, forked from `origin`.
        cudaSetDevice(unit[0]->device);
        bool ok = true;
        if (!b->origin)
            ok = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
        while (ok && (int)b->join.size() < nu) {
            cudaEvent_t e;
            ok = cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
            if (ok)
                b->join.push_back(e);
        }
        std::vector<uint64_t> before((size_t)nu);
        std::vector<int64_t> launched((size_t)nu);
        std::vector<IssueState> saved;
        for (int u = 0; u < nu; u++) {
            before[(size_t)u] = issue_digest(unit[(size_t)u]);
            launched[(size_t)u] = unit[(size_t)u]->launches;
            saved.emplace_back(unit[(size_t)u]);
        }
        ok = ok && cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        bool began = ok;
        ok = ok && cudaEventRecord(b->fork, b->origin) == cudaSuccess;
        for (int u = 0; ok && u < nu; u++)
            ok = cudaStreamWaitEvent(unit[(size_t)u]->stream, b->fork, 0) == cudaSuccess;
        for (int u : order)
            if (ok)
                ok = issue(u) == GENPK_OK;
        for (int u = 0; ok && u < nu; u++)
            ok = cudaEventRecord(b->join[(size_t)u], unit[(size_t)u]->stream) == cudaSuccess &&
                 cudaStreamWaitEvent(b->origin, b->join[(size_t)u], 0) == cudaSuccess;
        cudaGraph_t g = nullptr;
        if (began)
            ok = cudaStreamEndCapture(b->origin, &g) == cudaSuccess && ok;
        const bool cuda_ok = ok;
        b->graph_launches.assign((size_t)nu, 0);
        b->graph_deferred.assign((size_t)nu, genpk_ctx::Deferred{});
        for (int u = 0; u < nu; u++) {
            genpk_ctx *c = unit[(size_t)u];
            b->graph_launches[(size_t)u] = c->launches - launched[(size_t)u];
            c->launches = launched[(size_t)u];  // nothing ran yet
            b->graph_deferred[(size_t)u] = c->deferred;
            c->deferred.active = false;
        }
        // The call must leave every unit as it found it, so that each replay
        // starts from the state the capture started from.
        for (int u = 0; ok && u < nu; u++)
            ok = issue_digest(unit[(size_t)u]) == before[(size_t)u];
        if (ok)
            ok = cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess;
        if (ok)
            b->graph_attempts = 0;
        if (g)
            cudaGraphDestroy(g);
        b->graph_issued = issued;
        b->graph_digest = before;
        b->graph_grouped = grouped;
        if (!ok) {
            // Nothing ran: put back each unit's record of its device state and
            // run the call eagerly.  A call that did not leave the units as it
            // found them may do so the next time (a first pass allocates,
            // tunes, clears); a CUDA error during capture ends the graph path.
            cudaGetLastError();
            b->exec = nullptr;
            if (!cuda_ok || ++b->graph_attempts >= 3)
                b->graph_failed = true;
            for (int u = 0; u < nu; u++)
                saved[(size_t)u].restore(unit[(size_t)u]);
            std::fill(issued.begin(), issued.end(), false);
        }
    }
    if (b->exec) {
        cudaSetDevice(unit[0]->device);
        if (cudaGraphLaunch(b->exec, b->origin) != cudaSuccess ||
            cudaStreamSynchronize(b->origin) != cudaSuccess) {
            b->err = std::string("genpk_batch_power: graph replay failed: ") +
                     cudaGetErrorString(cudaGetLastError());
            drop_graph(b);
            return GENPK_ERR_CUDA;
        }
        b->replays++;
        for (int u = 0; u < nu; u++) {
            genpk_ctx *c = unit[(size_t)u];
            c->launches += b->graph_launches[(size_t)u];
            c->deferred = b->graph_deferred[(size_t)u];
        }
        issued = b->graph_issued;
    } else {
        for (int u : order)
            note_unit(u, issue(u));
    }
    std::vector<double> gp, gk;
    std::vector<int> gc;
    for (int u : order) {  // every issued unit is waited for, even after a failure
        if (!issued[(size_t)u])
            continue;
        genpk_ctx *c = unit[(size_t)u];
        cudaSetDevice(c->device);
        if (!grouped) {
            note(u, power_collect(c, power + (size_t)u * nrb,
                                  count ? count + (size_t)u * nrb : nullptr,
                                  keffs ? keffs + (size_t)u * nrb : nullptr));
            continue;
        }
        const genpk_batch::Group &g = b->groups[(size_t)u];
        const size_t nf = g.boxes.size();
        gp.assign(nf * nrb, 0.0);
        gc.assign((size_t)nrb, 0);
        gk.assign((size_t)nrb, 0.0);
        const int rc = power_collect(c, gp.data(), gc.data(), gk.data());
        note_unit(u, rc);
        for (size_t f = 0; f < nf; f++) {
            const int i = g.boxes[f];
            std::copy(gp.begin() + f * nrb, gp.begin() + (f + 1) * nrb, power + (size_t)i * nrb);
            if (count)
                std::copy(gc.begin(), gc.end(), count + (size_t)i * nrb);
            if (keffs)
                std::copy(gk.begin(), gk.end(), keffs + (size_t)i * nrb);
            if (g.bad_host[f])
                note_msg(GENPK_ERR_BAD_INPUT,
                         "box " + std::to_string(i) + ": " + std::to_string(g.bad_host[f]) +
                             " particle(s) with non-finite or out-of-range position/mass were "
                             "skipped");
        }
    }
    if (group_nomem && b->mode == GENPK_BATCH_AUTO) {
        // A group's scratch does not fit beside everything else: the automatic
        // mode runs per box from now on, starting with this call.
        b->mode = GENPK_BATCH_PER_BOX;
        drop_graph(b);
        b->have_last = false;
        b->err.clear();
        return genpk_batch_power(b, boxsize, pos, masses, mass, n, mass_norm, power, count, keffs);
    }
    b->last_mode = grouped ? GENPK_BATCH_GROUPED : GENPK_BATCH_PER_BOX;
    if (b->mode == GENPK_BATCH_AUTO && can_group && first == GENPK_OK && trial) {
        genpk_batch::AutoChoice &au = b->au;
        if (timed_slot >= 0)
            au.ms[timed_slot] = std::chrono::duration<double, std::milli>(
                                    std::chrono::steady_clock::now() - t_start)
                                    .count();
        if (++au.phase == 4)
            au.choice = au.ms[1] < au.ms[0] ? GENPK_BATCH_GROUPED : GENPK_BATCH_PER_BOX;
    }
    if (first == GENPK_OK)
        b->err.clear();
    return first;
}

int genpk_batch_auto_times(const genpk_batch *b, double *per_box_ms, double *grouped_ms)
{
    if (!b)
        return -1;
    if (per_box_ms)
        *per_box_ms = b->au.ms[0];
    if (grouped_ms)
        *grouped_ms = b->au.ms[1];
    return b->au.phase >= 4 ? b->au.choice : -1;
}

int genpk_inject_copy_timeout(genpk_ctx *ctx, int64_t chunk, int64_t wait_clocks)
{
    if (!ctx)
        return GENPK_ERR_INVALID;
    if (chunk < 0)
        return fail(ctx, GENPK_ERR_INVALID, "genpk_inject_copy_timeout: negative chunk");
    ctx->inject_chunk = chunk;
    ctx->inject_clocks = std::min<int64_t>(std::max<int64_t>(wait_clocks, 1024), (int64_t)1 << 31);
    return GENPK_OK;
}

}  // extern "C"
