/*
 * genpk_compat.h -- the reference's own hot-path signatures, backed by the GPU.
 *
 * libgenpk_compat.so exports fieldize(), invwindow() and powerspectrum() with
 * exactly the declarations of gen-pk.h:93,104,119 (fieldize keeps its C++
 * linkage, the other two are extern "C"), so gen-pk can link it in place of
 * fieldize.o and powerspectrum.o without touching the readers
 * (read_fieldize.cpp:90,333; read_fieldize_bigfile.cpp:121).
 *
 * Two modes per call:
 *  - bound:   the host grid pointer was registered with genpk_compat_bind();
 *             fieldize() then deposits into the context's device grid (the host
 *             array is not touched) and powerspectrum() on bound pointers runs
 *             the GPU FFT + binning, so the driver's fftw_execute calls can go.
 *  - unbound: plain reference semantics on host arrays: fieldize() adds the
 *             CIC density into `out`; powerspectrum() bins the caller's
 *             spectrum.  A private context per grid size is used.
 * Return value 0 = success, otherwise a genpk_status code.
 */
#ifndef GENPK_COMPAT_H
#define GENPK_COMPAT_H

#include <stdint.h>

#include "genpk_gb300.h"

#ifdef __cplusplus
/* gen-pk.h:93 (C++ linkage in the reference). */
int fieldize(double boxsize, int dims, double *out, int64_t segment_particles, float *positions,
             float *masses, double mass, int extra);
extern "C" {
#endif

/* gen-pk.h:104 */
double invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n);

/* gen-pk.h:119; fftw_complex is double[2]. */
int powerspectrum(int64_t dims, double (*outfield)[2], double (*outfield2)[2], int nrbins,
                  double *power, int *count, double *keffs, double total_mass,
                  double total_mass2);

/* Route fieldize()/powerspectrum() calls on host_field to grid `field` of ctx.
 * The binding also sets the first deposit to overwrite (like the driver's
 * memset at gen-pk.cpp:208).  Unbind before freeing ctx. */
int genpk_compat_bind(genpk_ctx *ctx, int field, const void *host_field);
int genpk_compat_unbind(const void *host_field);

/* Free the private contexts of unbound calls. */
void genpk_compat_release(void);

#ifdef __cplusplus
}
#endif
#endif /* GENPK_COMPAT_H */
