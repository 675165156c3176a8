/* Test infrastructure: the uniform generator linked into the reference's
 * marx2fits program (oracle/Makefile, target m2f) in place of jdmath's
 * JDMrandom (jdmath/src/random.c:151).  marx2fits draws uniforms for the
 * ACIS flight grade (compute_fltgrade, marx2fits.c:3864) and for
 * --pixadj=RANDOMIZE (compute_detxy, marx2fits.c:3707-3708); serving them
 * from a file lets the same uniforms drive the device pass.  The file named
 * by MXREF_UNIFORMS holds native-endian doubles, consumed in order; the
 * number drawn is printed to stderr at exit so that a fixture can check
 * that every event drew what it expected. */
#include <stdio.h>
#include <stdlib.h>

static FILE *g_fp;
static unsigned long g_drawn;

static void report(void) { fprintf(stderr, "mxref uniforms drawn: %lu\n", g_drawn); }

double JDMrandom(void) {
  double u;
  if (!g_fp) {
    const char *f = getenv("MXREF_UNIFORMS");
    if (!f || !(g_fp = fopen(f, "rb"))) {
      fprintf(stderr, "MXREF_UNIFORMS does not name a readable file\n");
      exit(3);
    }
    atexit(report);
  }
  if (fread(&u, sizeof u, 1, g_fp) != 1) {
    fprintf(stderr, "MXREF_UNIFORMS exhausted after %lu draws\n", g_drawn);
    exit(3);
  }
  g_drawn++;
  return u;
}
