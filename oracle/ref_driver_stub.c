/* Link-time stand-in for the reference's picture writer, which its Bloch
 * driver references from its visualisation branches (never taken with
 * maxwell_visualization=n).  The driver is built without Cairo, so the
 * writer is absent from edge2d.c; this version draws nothing. */
#include "edge2d.h"

void cairodraw_edge2d(const edge2d *x, int gx, int gy, const epspattern *pat, const char *filename);

void
cairodraw_edge2d(const edge2d *x, int gx, int gy, const epspattern *pat, const char *filename)
{
  (void) x; (void) gx; (void) gy; (void) pat; (void) filename;
}
