/* Pre-included when compiling the GCGE-1.0 sources for the oracle/_ref build.
 * Defines the reference's configuration macros (src/gcge_config.h) with MPI
 * switched off; the reference header's include guard then skips its own copy.
 * Test infrastructure only. */
#ifndef _GCGE_CONFIG_H_
#define _GCGE_CONFIG_H_
#include <float.h>
#define GCGE_DOUBLE double
#define GCGE_INT int
#define GET_PART_TIME 1
#define GCGE_USE_MPI 0
#endif
