/* Build configuration for compiling the reference engine's CPU/BLAS
 * evaluation path as a test oracle.  It is force-included (-include) ahead
 * of every reference translation unit.  It defines CONFIG_INCLUDED so that
 * the reference's own config.h becomes a no-op, and selects the BLAS
 * backend (USE_BLAS + USE_OPENBLAS) instead of OpenCL.  The remaining
 * definitions are the ones the reference expects from its config.h
 * (config.h:1-79): timing source, CPU limit and the fixed-width integer
 * typedefs. */
#ifndef CONFIG_INCLUDED
#define CONFIG_INCLUDED
#define HAVE_SELECT
#define GETTIMEOFDAY
#define USE_OPTIONS
#define USE_BLAS
#define USE_OPENBLAS
#define USE_SEARCH
#define PROGRAM_NAME "Leela"
#define PROGRAM_VERSION "0.11.0"
#define MAX_CPUS 64
typedef int int32;
typedef short int16;
typedef signed char int8;
typedef unsigned int uint32;
typedef unsigned short uint16;
typedef unsigned char uint8;
typedef long long int int64;
typedef unsigned long long int uint64;
#include <sys/time.h>
#include <time.h>
typedef struct timeval rtime_t;
#endif
