/* C-linkage entry points for the reference's own fieldize() (C++ linkage,
 * gen-pk.h:93) so the test oracle can load it with ctypes.  Only used to
 * build oracle/_ref/libgenpk_ref.so from the reference sources. */
#include <cstdint>
int fieldize(double boxsize, int dims, double *out, int64_t segment_particles,
             float *positions, float *masses, double mass, int extra);
extern "C" int ref_fieldize(double boxsize, int dims, double *out, int64_t n,
                            float *pos, float *masses, double mass, int extra)
{
    return fieldize(boxsize, dims, out, n, pos, masses, mass, extra);
}
