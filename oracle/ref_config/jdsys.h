/* Host description that the reference's jdmath build would otherwise
 * generate by running its sysconf probe: type sizes for LP64 and the byte
 * order of a little-endian host (its data files are big-endian). */
#ifndef INT16_DEFINED
#define INT16_DEFINED
#define SIZEOF_SHORT	2
#define SIZEOF_INT	4
#define SIZEOF_LONG	8
#define SIZEOF_FLOAT	4
#define SIZEOF_DOUBLE	8
#define NEEDS_BYTE_SWAP
#endif /* INT16_DEFINED */
