/* rc_gb300 -- the MS5 pipeline's kernel bindings (librc_gb300_ms5.so).
 *
 * MS5 and MS6 bind two symbols under the same names with different
 * signatures or semantics, so the MS5 variant is a separate build of the same
 * sources (rc_gb300.build(ms5=True), compiled with -DGB_MS5_ABI).  It exports
 * everything include/rc_gb300.h declares except MS6's kern_scatter and
 * kern_fft, which it replaces by the two below.  MS5's kern_init, kern_detile
 * and kern_rotate are MS6's (MS5/kernel/cpu/gridding/{init,detile,rotate}.cpp
 * equal MS6's).
 */
#ifndef RC_GB300_MS5_H
#define RC_GB300_MS5_H

#include "rc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifdef GB_MS5_ABI
/* replaces the kernel MS5/kernel/cpu/gridding/scatter.cpp:10-121 generates,
 * bound by MS5/programs/Kernel/Gridder.hs:28-35: grid += vis * gcf with the
 * GCF size fixed at 16 ((2,16,16,64) doubles) and no margin argument; a
 * visibility is kept when its corner lies in min .. min + extent - 16 - 1 of
 * the grid buffer.  GB_ERR_ARG for any other GCF size or a malformed buffer. */
int kern_scatter(double scale, int32_t grid_size, buffer_t *vis, buffer_t *gcf, buffer_t *uvg);

/* replaces the kernel MS5/kernel/cpu/gridding/fft.cpp:540-605 generates, bound
 * by MS5/programs/Kernel/FFT.hs:15-16: grid (2,2048,2048) -> real image
 * (2048,2048), the inverse pipeline of MS6's kern_ifft with the grid
 * hermitised without the 1/2 and the image not divided by n (2 n times
 * kern_ifft's image).  GB_ERR_ARG for another size. */
int kern_fft(buffer_t *uvg, buffer_t *img);
#endif

#ifdef __cplusplus
}
#endif

#endif
