/* No-op stand-in for the Cairo header so that the reference's grid2d.c
 * compiles in a container without Cairo.  Drawing is outside the
 * eigensolver path; every function here does nothing. */
#ifndef ORACLE_REF_STUB_CAIRO_H
#define ORACLE_REF_STUB_CAIRO_H
typedef struct { int unused; } cairo_t;
typedef struct { int unused; } cairo_surface_t;
#define CAIRO_FORMAT_RGB24 1
static inline cairo_surface_t *cairo_image_surface_create(int f, double w, double h) { (void) f; (void) w; (void) h; return 0; }
static inline cairo_t *cairo_create(cairo_surface_t *s) { (void) s; return 0; }
static inline void cairo_scale(cairo_t *c, double x, double y) { (void) c; (void) x; (void) y; }
static inline void cairo_set_line_width(cairo_t *c, double w) { (void) c; (void) w; }
static inline void cairo_surface_destroy(cairo_surface_t *s) { (void) s; }
static inline void cairo_rectangle(cairo_t *c, double x, double y, double w, double h) { (void) c; (void) x; (void) y; (void) w; (void) h; }
static inline void cairo_set_source_rgb(cairo_t *c, double r, double g, double b) { (void) c; (void) r; (void) g; (void) b; }
static inline void cairo_fill(cairo_t *c) { (void) c; }
static inline int cairo_surface_write_to_png(cairo_surface_t *s, const char *f) { (void) s; (void) f; return 0; }
static inline void cairo_destroy(cairo_t *c) { (void) c; }
#endif
