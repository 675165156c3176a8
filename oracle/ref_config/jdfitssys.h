/* Same host description for the reference's FITS library, which would
 * otherwise generate it with its own sysconf probe. */
#include "jdsys.h"
