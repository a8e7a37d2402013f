/* Minimal stand-in for <fftw3.h>, used only to compile the reference's
 * fieldize.cpp and powerspectrum.c into the test oracle (oracle/_ref).
 * Those two files need nothing from FFTW but the fftw_complex type, which
 * FFTW defines as an array of two doubles (re, im). */
#ifndef ORACLE_SHIM_FFTW3_H
#define ORACLE_SHIM_FFTW3_H
typedef double fftw_complex[2];
#endif
