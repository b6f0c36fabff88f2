/* Stub bodies for the fftw3.h stand-in (see that header).  fftw_malloc/free are
 * real; everything else aborts with a message. */
#include "fftw3.h"
#include <stdlib.h>

void *fftw_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 64) != 0) return NULL;
  return p;
}
void fftw_free(void *p) { free(p); }

static void die(const char *what) {
  fprintf(stderr, "oracle fftw shim: %s needs FFTW, which is not available\n", what);
  abort();
}
fftw_plan fftw_plan_r2r_1d(int n, double *i, double *o, fftw_r2r_kind k, unsigned f) {
  (void)n; (void)i; (void)o; (void)k; (void)f; die("fftw_plan_r2r_1d"); return NULL;
}
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double *i, double *o, fftw_r2r_kind k0,
                           fftw_r2r_kind k1, unsigned f) {
  (void)n0; (void)n1; (void)i; (void)o; (void)k0; (void)k1; (void)f;
  die("fftw_plan_r2r_2d"); return NULL;
}
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *i, fftw_complex *o, int s, unsigned f) {
  (void)n; (void)i; (void)o; (void)s; (void)f; die("fftw_plan_dft_1d"); return NULL;
}
void fftw_execute(const fftw_plan p) { (void)p; die("fftw_execute"); }
void fftw_destroy_plan(fftw_plan p) { (void)p; }
void fftw_flops(const fftw_plan p, double *a, double *m, double *f) {
  (void)p; (void)a; (void)m; (void)f; die("fftw_flops");
}
void fftw_print_plan(const fftw_plan p) { (void)p; die("fftw_print_plan"); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup(void) {}
void fftw_cleanup_threads(void) {}
int fftw_import_wisdom_from_filename(const char *f) { (void)f; return 0; }
int fftw_export_wisdom_to_filename(const char *f) { (void)f; return 0; }
