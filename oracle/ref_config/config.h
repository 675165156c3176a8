/* Platform description used to compile the reference's own C sources
 * directly with gcc (no configure step).  It stands in for the header that
 * the reference's autoconf build would write from each library's config.hin;
 * every value is a fact about LP64 Linux with glibc (x86_64 here). */
#ifndef MX_REF_CONFIG_H
#define MX_REF_CONFIG_H
#define HAVE_STDLIB_H 1
#define HAVE_UNISTD_H 1
#define HAVE_LIMITS_H 1
#define HAVE_TIMEGM 1
#define SIZEOF_SHORT 2
#define SIZEOF_INT 4
#define SIZEOF_LONG 8
#define SIZEOF_FLOAT 4
#define SIZEOF_DOUBLE 8
#define HAVE_ISNAN 1
#define HAVE_ISINF 1
#define HAVE_FINITE 1
#define HAVE_ERF 1
#define HAVE_FSEEKO 1
#define FSEEK(a,b,c) fseeko(a,b,c)
#define FTELL(a) ftello(a)
#endif
