/*
 * genpk_gb300.h -- C ABI of the GB300 (sm_103a) power-spectrum hot path.
 *
 * This library replaces GenPK's CIC deposit, FFT and binning calls:
 *
 *   reference call                                 replaced by
 *   ---------------------------------------------  -----------------------------
 *   fftw_malloc + fftw_plan_dft_r2c_3d             genpk_ctx_create
 *     (gen-pk.cpp:176-193, :263-270, :314-321)
 *   memset(field, 0, ...) (gen-pk.cpp:208,267)     genpk_zero
 *   fieldize() (gen-pk.h:93, fieldize.cpp:46)      genpk_deposit
 *     called from read_fieldize.cpp:90,333 and
 *     read_fieldize_bigfile.cpp:121
 *   fftw_execute + powerspectrum()                 genpk_power
 *     (gen-pk.cpp:233-234, :295-297, :345-348;
 *      gen-pk.h:119, powerspectrum.c:35)
 *   invwindow() (gen-pk.h:104, fieldize.cpp:125)   genpk_invwindow
 *   fftw_free / fftw_destroy_plan                  genpk_ctx_destroy
 *     (gen-pk.cpp:363-364)
 *
 * and adds what the reference does not have: batched multi-field spectra
 * (genpk_power_multi) and the adjoint of a P(k) loss (genpk_adjoint).
 *
 * Conventions
 *  - Every function returns a genpk_status; nothing aborts, exits or asserts.
 *    genpk_last_error(ctx) gives a message for the last failure on ctx.
 *  - Grids live on the GPU.  A context owns `nfields` FP32 grids of
 *    dims x dims x 2*(dims/2+1) floats: the in-place r2c layout FFTW and cuFFT
 *    share (gen-pk.cpp:176), x slowest, z fastest.
 *  - Particle pointers may be host or device memory.  Host buffers are copied
 *    before genpk_deposit returns, so the caller may free them at once, as
 *    read_fieldize does.  Device buffers are read in stream order on the
 *    context's stream and must stay valid until genpk_sync or the next
 *    genpk_power on that context.
 *  - Output arrays of genpk_power* and genpk_adjoint are host memory unless a
 *    function says otherwise.  Results are complete when the call returns.
 *  - One context per host thread; a context is not thread-safe.  Different
 *    contexts may be used from different host threads at the same time (each
 *    has its own stream): their work overlaps on the GPU and the results equal
 *    those of the contexts run one at a time.
 */
#ifndef GENPK_GB300_H
#define GENPK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct genpk_ctx genpk_ctx;

typedef enum genpk_status {
    GENPK_OK = 0,
    GENPK_ERR_INVALID = 1,     /* bad argument (null pointer, field index, dims ...) */
    GENPK_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    GENPK_ERR_CUFFT = 3,       /* a cuFFT call failed */
    GENPK_ERR_NOMEM = 4,       /* device or pinned-host allocation failed */
    GENPK_ERR_BAD_INPUT = 5,   /* non-finite or out-of-range particle data seen on the GPU */
    GENPK_ERR_STATE = 6,       /* call not valid in the field's current state */
    GENPK_ERR_UNSUPPORTED = 7, /* size or option this build does not handle */
    GENPK_ERR_TIMEOUT = 8      /* a bounded device-side wait gave up */
} genpk_status;

/* genpk_ctx_create flags */
#define GENPK_FLAG_TIMING 0x1u       /* record per-stage CUDA-event times */
#define GENPK_FLAG_DETERMINISTIC 0x2u /* reserved: all reductions are already ordered */

/* Create a context for dims^3 grids, nrbins log-k bins and nfields grids.
 * Builds the bin tables (the reference's bin expression, powerspectrum.c:38,66)
 * and cuFFT plans, and allocates the grids.  dims >= 2, 1 <= nrbins,
 * 1 <= nfields <= GENPK_MAX_FIELDS. */
#define GENPK_MAX_FIELDS 8
int genpk_ctx_create(int64_t dims, int nrbins, int nfields, unsigned flags, genpk_ctx **out);

/* Free every device resource of ctx.  Accepts NULL. */
void genpk_ctx_destroy(genpk_ctx *ctx);

/* Message for the last error on ctx (never NULL; "" after success). */
const char *genpk_last_error(const genpk_ctx *ctx);

/* Text for a status code. */
const char *genpk_status_string(int status);

/* Empty a grid: replaces memset(field,0,...) (gen-pk.cpp:208).  Lazy: the next
 * deposit writes the grid instead of adding to it. */
int genpk_zero(genpk_ctx *ctx, int field);

/* CIC-deposit n particles into grid `field` with += semantics, as
 * fieldize(boxsize, dims, field, n, pos, masses, mass, 1) does
 * (fieldize.cpp:46-113): pos is float[n][3] in box units, masses float[n] or
 * NULL for a uniform `mass`.  Periodic wrap.  May be called many times per
 * field (reader chunks, several files, stars added to gas).  Host-pointer
 * deposits are staged on the GPU and deposited in as few passes as staging
 * memory allows; the deposited density is mean-subtracted on the GPU (only the
 * excluded k=0 mode changes). */
int genpk_deposit(genpk_ctx *ctx, int field, double boxsize, const float *pos,
                  const float *masses, double mass, int64_t n);

/* fftw_execute + powerspectrum for one pair of grids (A == B: auto spectrum).
 * Runs the r2c FFT of each grid still in density form (in place), then the
 * fused deconvolution + log-k binning.  power[nrbins], count[nrbins],
 * keffs[nrbins] have the meaning and normalisation of powerspectrum.c:35-111:
 * power /= mass_a*mass_b*count, keffs /= count, zero where count == 0. */
int genpk_power(genpk_ctx *ctx, int field_a, int field_b, double mass_a, double mass_b,
                double *power, int *count, double *keffs);

/* Several spectra in one pass over the modes.  fields[nf] are FFT'd in one
 * batched plan where they are still densities; pairs[2*np] index into the
 * context's grids; pair_mass[2*np] are the two normalisation masses of each
 * pair.  power is [np][nrbins]; count and keffs are [nrbins] (shared by all
 * pairs, they depend only on the grid).  Replaces the per-type loop of
 * gen-pk.cpp:204-239 and the cross-spectrum branches :240-356. */
int genpk_power_multi(genpk_ctx *ctx, int np, const int *pairs, const double *pair_mass,
                      double *power, int *count, double *keffs);

/* One whole step of the per-species loop: fields 0..nspecies-1 are cleared,
 * species s (n[s] particles pos[s], masses[s] or the uniform mass[s]) is
 * deposited into field s, and the spectra pairs[2*np] (field indices below
 * nspecies, normalisation masses pair_mass[2*np]) come back as
 * genpk_power_multi returns them.  The gen-pk loop of gen-pk.cpp:204-356 (one
 * fieldize per type, the FFTs, powerspectrum per auto and cross pair) in one
 * call.  Repeated calls with the same arguments (the same arrays, counts,
 * masses and pairs; the arrays' contents may change) replay a CUDA graph of
 * the whole step, captured on the second such call, when every array is in
 * device memory and the context has no GENPK_FLAG_TIMING: the same results
 * bit for bit, one launch per step.  Any other use of the context between
 * steps drops the graph (the next identical step captures it again). */
int genpk_power_step(genpk_ctx *ctx, int nspecies, double boxsize, const float *const *pos,
                     const float *const *masses, const double *mass, const int64_t *n, int np,
                     const int *pairs, const double *pair_mass, double *power, int *count,
                     double *keffs);

/* Graphs for genpk_power_step on (1, the default) or off (0; drops one). */
int genpk_power_step_use_graph(genpk_ctx *ctx, int on);

/* genpk_power_step calls served by a graph replay, or -1 for a null ctx. */
int64_t genpk_power_step_replays(const genpk_ctx *ctx);

/* The reference's inverse CIC window, fieldize.cpp:125-133 (host function). */
double genpk_invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n);

/* Host-only: the weighted mode count and mean |k| of every bin for a dims^3
 * grid and nrbins bins -- the count[] and keffs[] powerspectrum() returns
 * (powerspectrum.c:55-108), which depend only on the grid.  Needs no GPU. */
int genpk_geometry(int64_t dims, int nrbins, int *count, double *keffs);

/* Load a caller-computed half-complex spectrum (dims*dims*(dims/2+1) complex
 * values as interleaved float64 re, im -- FFTW's in-place r2c output,
 * gen-pk.cpp:185) into grid `field`, so genpk_power bins it without an FFT.
 * This is the path behind the reference-signature powerspectrum() drop-in. */
int genpk_load_spectrum(genpk_ctx *ctx, int field, const double *spectrum);

/* Bin index the library assigns to integer |k|^2 = kk2 on ctx's grid; the
 * reference's floor(binsperunit*log(sqrt(kk2))) (powerspectrum.c:38,66). */
int genpk_bin_of(const genpk_ctx *ctx, int64_t kk2);

/* Wait for all work on ctx and report device-side input errors. */
int genpk_sync(genpk_ctx *ctx);

/* Copy grid `field` (density form) to host as float64 padded grid
 * (dims*dims*2*(dims/2+1)), the same array fieldize() would have produced.
 * Intended for tests; flushes pending deposits. */
int genpk_read_field(genpk_ctx *ctx, int field, double *out);

/* Gradient of a P(k) loss with respect to particle positions and masses
 * (no reference counterpart).  For the auto spectrum of grid `field` built from
 * the n particles (pos, masses|NULL, mass) with normalisation mass_norm:
 * given dl_dp[nrbins] = dL/dP_b, writes grad_pos[n][3] = dL/dpos and, when
 * masses != NULL, grad_mass[n] = dL/dm (including the dependence of mass_norm
 * on the masses, d mass_norm / d m_p = 1).  *dl_dmass_norm receives dL/dM.
 * If the grid still holds this species' spectrum (after genpk_power) it is
 * reused; otherwise, or with recompute != 0, the density is re-deposited and
 * transformed again.  pos/masses/grad_* may be host or device pointers (all
 * of one kind). */
int genpk_adjoint(genpk_ctx *ctx, int field, double boxsize, const float *pos,
                  const float *masses, double mass, int64_t n, double mass_norm,
                  const double *dl_dp, float *grad_pos, float *grad_mass,
                  double *dl_dmass_norm, int recompute);

/* Per-kernel / per-stage device times (milliseconds, CUDA events on the
 * context's stream) of all work issued since the last genpk_timing_reset, when
 * the context was created with GENPK_FLAG_TIMING.  names[i] point at static
 * strings (e.g. "dep_tile", "fft", "bin").  Waits for that work.  Returns the
 * number of intervals written (<= cap). */
int genpk_stage_times(const genpk_ctx *ctx, const char **names, float *ms, int cap);

/* Start a new timing window (see genpk_stage_times). */
int genpk_timing_reset(genpk_ctx *ctx);

/* The sorted engine's configuration: that of its latest pass (tile edge
 * lengths and sort CTA count), or before any pass the default. */
int genpk_deposit_config(const genpk_ctx *ctx, int *tile_x, int *tile_y, int *tile_z,
                         int *sort_ctas);

/* The deposit autotuner, for passes whose particle order has no spatial
 * coherence: on the first clean pass of each particle density band (half
 * octaves of particles per cell) and mass kind, the pass runs twice per
 * candidate -- the sorted engine with tiles 8^3, 16x16x8 and 16^3, each with
 * 1 and 2 sort CTAs per SM, and, when the engine is automatic,
 * the stream engine -- timed with CUDA events, and the fastest is kept for
 * that band.  Every candidate writes the same grid.  This returns the latest
 * tuning's trials (at most cap, the number written): tile edges (0 x 0 x 0
 * for the stream engine), sort CTA count (0 for the stream engine) and
 * milliseconds each.  No reference counterpart (the reference's deposit has
 * no tunable). */
int genpk_deposit_trials(const genpk_ctx *ctx, int *tile_x, int *tile_y, int *tile_z,
                         int *sort_ctas, float *ms, int cap);

/* Fix the deposit tile of the sorted engine (cells per edge; supported:
 * 8^3, 16x16x8 and 16^3), which turns its autotuner off; (0, 0, 0) turns it
 * back on.  The sorted engine's grid does not depend on the tile. */
int genpk_set_deposit_tile(genpk_ctx *ctx, int tile_x, int tile_y, int tile_z);

/* Deposit engines.  All three add the same integer CIC weights exactly (64-bit
 * fixed point) and round each cell once: their grids are bit-identical and do
 * not depend on particle order.
 *  SORTED: counting sort into cell tiles, shared-memory tile sums; any order.
 *  WINDOW: for spatially coherent particle order (lattice or Peano-Hilbert
 *          order of most snapshots): per-chunk shared windows, no sort.
 *  STREAM: the window engine's chunk pipeline without windows: reductions
 *          straight to the accumulator, merged between neighbouring particles
 *          of one z cell column; for coherent order at about one particle per
 *          cell, where windows merge few adds.
 *  AUTO (default): from a sample of particle chunks, STREAM or WINDOW when the
 *          order is coherent (by window cells per particle), else SORTED. */
#define GENPK_ENGINE_AUTO 0
#define GENPK_ENGINE_SORTED 1
#define GENPK_ENGINE_WINDOW 2
#define GENPK_ENGINE_STREAM 3
int genpk_set_deposit_engine(genpk_ctx *ctx, int engine);

/* Engine the most recent deposit pass used (GENPK_ENGINE_SORTED, _WINDOW or
 * _STREAM). */
int genpk_last_deposit_engine(const genpk_ctx *ctx);

/* Forward-FFT path (replaces the driver-owned FFTW plan, gen-pk.cpp:186-193,233).
 *  AUTO (default): for power-of-two N in [64, 512], a batched 2-D cuFFT R2C
 *          over the x-planes, then the library's own x-axis pass, which also
 *          bins a single auto spectrum in the same read of the spectrum; other
 *          N use CUFFT3D.
 *  CUFFT3D: one 3-D cuFFT R2C, then the binning kernel.
 * Both leave the same half-complex spectrum in the grid. */
#define GENPK_FFT_AUTO 0
#define GENPK_FFT_CUFFT3D 1
int genpk_set_fft_mode(genpk_ctx *ctx, int mode);

/* Number of kernels the library launched on ctx since creation. */
int64_t genpk_kernel_launches(const genpk_ctx *ctx);

/* Many independent boxes in one call -- the per-type loop of
 * gen-pk.cpp:204-239 generalised to a batch of snapshots or boxes with
 * different grids.  Box b has a dims[b]^3 grid; all boxes share nrbins.
 * Every box has a context of its own (grid, accumulator, stream).  Errors as
 * for genpk_ctx_create; genpk_batch_last_error explains them. */
typedef struct genpk_batch genpk_batch;
int genpk_batch_create(int nboxes, const int64_t *dims, int nrbins, unsigned flags,
                       genpk_batch **out);
void genpk_batch_destroy(genpk_batch *b);
const char *genpk_batch_last_error(const genpk_batch *b);

/* The auto spectrum of every box: its n[b] particles pos[b] (float[n][3]),
 * masses[b] (float[n]) or NULL (masses itself may be NULL) for the uniform
 * mass[b], normalised by mass_norm[b] (powerspectrum.c:102-108).  power,
 * count and keffs are [nboxes][nrbins] host arrays (count and keffs may be
 * NULL).  One host thread issues all the work, per box or grouped by grid
 * size (genpk_batch_set_mode; by default whichever timed faster), then waits
 * once per box or group for the results (a repeated call replays a captured
 * CUDA graph of all of it: genpk_batch_use_graph).  Per box, every box's
 * deposit, transform and binning run on its own stream, largest box first, so
 * that the boxes overlap on the GPU, and the deposit engine of each box is
 * chosen as genpk_deposit chooses it (and remembered for the same arrays).
 * Particle arrays may be host or device memory; pinned host and device
 * arrays are read while other work runs and must stay valid until the call
 * returns.  Returns the first failure (the message names the box); all
 * issued work is still waited for. */
int genpk_batch_power(genpk_batch *b, const double *boxsize, const float *const *pos,
                      const float *const *masses, const double *mass, const int64_t *n,
                      const double *mass_norm, double *power, int *count, double *keffs);

/* Box i's context (for its stage times, engine and configuration), or NULL. */
genpk_ctx *genpk_batch_box(genpk_batch *b, int i);

/* Kernels launched by all the batch's boxes and groups since creation (a
 * graph replay counts the kernels it launches). */
int64_t genpk_batch_launches(const genpk_batch *b);

/* CUDA graph of a whole call (on by default).  The second of two
 * consecutive genpk_batch_power calls with the same arguments (the same
 * arrays, counts, box sizes and masses; the arrays' contents may change) is
 * captured: the work of every box (or group) is forked from one stream onto
 * their streams and joined back.  Later identical calls replay the graph with
 * one launch; results are identical to the eager path's, bit for bit.  A call
 * with other arguments runs eagerly and drops the graph, and so does any use
 * of a box's context on its own between calls.  The capture is kept only if
 * the call leaves every context's state as it found it; otherwise the call runs
 * eagerly and a later identical call tries again (three tries; a CUDA error
 * during capture ends the graph path).  Boxes created with GENPK_FLAG_TIMING
 * always run eagerly (stage events are not re-recorded by a replay).
 * on = 0 turns graphs off (and drops one), 1 turns them back on. */
int genpk_batch_use_graph(genpk_batch *b, int on);

/* Calls served by a graph replay since creation, or -1 for a null batch. */
int64_t genpk_batch_graph_replays(const genpk_batch *b);

/* How genpk_batch_power issues the boxes.
 * GENPK_BATCH_PER_BOX: each box has its own deposit pass (its engine chosen
 * as genpk_deposit chooses it), transform and binning.
 * GENPK_BATCH_GROUPED: the boxes that share a grid size (up to 32; more make
 * further groups) are the fields of one internal context and go through one
 * grouped sorted-engine pass -- one launch of each kernel of the pass for all
 * of them: the sort CTAs shared out over the boxes' particles by a table of
 * (box, particle range, record range), the per-tile kernels indexed by box --
 * with a tile shape and sort CTAs per SM tuned per group on its first call
 * (trials as for genpk_deposit_trials, on the group's context); then one
 * batched 2-D R2C over every x-plane of the group, and one x pass that bins
 * every box's auto spectrum (a histogram per box).  A call qualifies when
 * every array is in device memory, every argument is valid, every grid's
 * tile histogram fits in shared memory (40960 tiles of 16^3 cells: grids up
 * to 544 cells a side) and the boxes of a grid size hold fewer than 2^32
 * particles; any other call runs per box.  The grids are the per-box sorted engine's bit for
 * bit; the spectra agree with the per-box path's to FP32 transform rounding.
 * A skipped particle is reported for its box.
 * GENPK_BATCH_AUTO (the default): for calls that qualify, the faster of the
 * two for calls of the same shape (particle counts and mass kinds): the first
 * four such calls run per box, grouped, per box and grouped (the first two
 * tune; the last two are timed by wall clock, and none is captured), later
 * calls the faster way (the per-box path keeps the stream and window engines
 * for spatially ordered boxes; the grouped pass sorts every box).  A call of
 * another shape starts the trials again.  Where the groups' contexts or their
 * scratch cannot be allocated, the automatic mode runs per box from then on,
 * starting with that call (the grouped mode returns GENPK_ERR_NOMEM).
 * Switching modes drops a captured graph. */
#define GENPK_BATCH_PER_BOX 0
#define GENPK_BATCH_GROUPED 1
#define GENPK_BATCH_AUTO 2
int genpk_batch_set_mode(genpk_batch *b, int mode);

/* The way the latest call ran (GENPK_BATCH_PER_BOX or GENPK_BATCH_GROUPED),
 * or -1 before the first call or for a null batch. */
int genpk_batch_last_mode(const genpk_batch *b);

/* GENPK_BATCH_AUTO's timed trial calls of the current shape (ms, 0 where not
 * run yet) and its choice, or -1 while the trials run (or for a null batch). */
int genpk_batch_auto_times(const genpk_batch *b, double *per_box_ms, double *grouped_ms);

/* Groups made by the first grouped call (0 before it), or -1 for a null
 * batch. */
int genpk_batch_groups(const genpk_batch *b);

/* Group g's context (for its kernel launches, genpk_deposit_config and
 * genpk_deposit_trials), or NULL.  nboxes (may be NULL) receives its number
 * of boxes (at most 32) and boxes (may be NULL, else room for 32) their batch
 * indices, field 0 first. */
genpk_ctx *genpk_batch_group(genpk_batch *b, int g, int *nboxes, int *boxes);

/* Testing aid for the bounded device waits (no reference counterpart; the
 * reference has no device code).  The next window- or stream-engine deposit
 * pass on ctx does not issue the bulk copy of its chunk number `chunk`
 * (chunks of the pass's chunk length, 4096 particles in the stream mode,
 * counted from 0 in particle order), so the kernel's bounded wait for that
 * copy gives up after wait_clocks SM clocks (clamped to [1024, 2^31]).  The
 * CTA then loads that chunk and its later ones with plain loads, so the grid
 * is still complete, and the next sync point (genpk_sync, genpk_power)
 * returns GENPK_ERR_TIMEOUT.  Nothing faults or hangs and the context stays
 * usable.  Applies to one pass; a pass of the sorted engine ignores it. */
int genpk_inject_copy_timeout(genpk_ctx *ctx, int64_t chunk, int64_t wait_clocks);

/* Largest sizes genpk_power_noalloc accepts. */
#define GENPK_NOALLOC_MAX_DIMS 1024
#define GENPK_NOALLOC_MAX_NRBINS 1024

/* Deconvolution + log-k binning of a spectrum already on the GPU, without
 * allocating any memory.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- code running under an allocator that
 * owns the device, or a loop that cannot afford an allocation's implicit
 * synchronisation -- and so cannot create a genpk_ctx.
 *
 * spectrum_a / spectrum_b: device pointers to FP32 half-complex spectra of a
 *   dims^3 grid in the in-place r2c layout (dims*dims*(dims/2+1) interleaved
 *   re, im pairs, rows of dims/2+1 complex values); spectrum_b may be NULL or
 *   equal to spectrum_a for an auto spectrum.
 * power: device pointer, nrbins doubles, written in stream order.
 * count, keffs: host arrays of nrbins (may be NULL), filled before returning.
 * stream: a cudaStream_t, or NULL for the default stream.
 * Same normalisation as genpk_power; the last bin uses the spectrum's own
 * (k = N/2, N/2, N/2) value.  dims <= GENPK_NOALLOC_MAX_DIMS and
 * nrbins <= GENPK_NOALLOC_MAX_NRBINS, else GENPK_ERR_UNSUPPORTED.
 *
 * Its scratch (about 2.5 MB: bin tables and per-block partial sums) is a
 * static array in the library's device image, held by every GPU that loads the
 * library until the process exits.  The first call on each device looks up
 * the array's device address; with CUDA's lazy module loading (the default)
 * that lookup is what loads the module and reserves the array, so it can fail
 * (GENPK_ERR_CUDA) once an allocator has claimed the whole device: make one
 * call on each device before the allocator takes it.  A call with a
 * (dims, nrbins) other than the previous call's on that device also rebuilds
 * the bin tables on the host and copies them to the array on `stream`.
 * Every call shares the array and keeps its last contents, so calls that
 * overlap on the GPU race; serialise them. */
int genpk_power_noalloc(const float *spectrum_a, const float *spectrum_b, int64_t dims,
                        int nrbins, double mass_a, double mass_b, double *power, int *count,
                        double *keffs, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GENPK_GB300_H */
