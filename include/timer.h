/* Wall-clock helper of the reference (libgpufs/timer.h:24): microseconds. */
#ifndef TIMER
#define TIMER
#include <sys/time.h>
#ifdef __cplusplus
extern "C"
#endif
    double
    _timestamp(void);
#endif
