/* Project-written stand-in for the FFTW2 single-precision types the reference uses
 * on its hot path (powerspectrum.h:5-14, interface_gadget.h:13-21): only the element
 * types; no transform is needed.  Test infrastructure: not shipped. */
#ifndef KSP_SHIM_SFFTW_H
#define KSP_SHIM_SFFTW_H
typedef float fftw_real;
typedef struct { fftw_real re, im; } fftw_complex;
#endif
