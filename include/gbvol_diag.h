/* gbvol_diag.h -- diagnostic entry points of the GB300 structured-volume
 * library.  A renderer user needs none of them: the test suite uses them to
 * check that the device's angle routines (bounded sine/cosine, arc cosine,
 * arc tangent), which the renderer uses where the reference calls libm,
 * give the host's results bit for bit and stay within their error bounds.
 * No counterpart in the reference.  Same conventions as gbvol.h.
 */
#ifndef GBVOL_DIAG_H
#define GBVOL_DIAG_H
#include "gbvol.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The renderer's bounded sine/cosine (angles in [-pi/4, 2pi + pi/4]) for n
   arguments: on the host (on_device = 0; host pointers) or in a kernel on
   `stream` (on_device = 1; device pointers).  Both give identical results;
   tests check them against float64 sine and cosine. */
gbv_status gbv_selftest_sincos(const float *x, long long n, float *sn,
                               float *cs, int on_device, void *stream);

/* The renderer's arc cosine and two-argument arc tangent of env-map angles:
   acos_x[i] = acos(x[i]) (x in [-1, 1]) and atan2_yx[i] = atan2(y[i], x[i]),
   on the host (on_device = 0; host pointers) or in a kernel on `stream`
   (on_device = 1; device pointers).  Both give identical results; tests
   check them against float64. */
gbv_status gbv_selftest_angles(const float *y, const float *x, long long n,
                               float *acos_x, float *atan2_yx, int on_device,
                               void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBVOL_DIAG_H */
