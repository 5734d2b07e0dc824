/* No-op stand-in for the Cairo PDF header (see cairo.h in this folder). */
#ifndef ORACLE_REF_STUB_CAIRO_PDF_H
#define ORACLE_REF_STUB_CAIRO_PDF_H
#include "cairo.h"
static inline cairo_surface_t *cairo_pdf_surface_create(const char *f, double w, double h) { (void) f; (void) w; (void) h; return 0; }
#endif
