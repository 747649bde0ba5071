// lib/time_util.h -- wall clock in seconds, as the reference's rtclock
// (lib/time_util.cpp:3-11) returns it.
#ifndef LIB_TIME_UTIL_
#define LIB_TIME_UTIL_
#include <stdio.h>
#include <sys/time.h>

static inline double rtclock()
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + tv.tv_usec * 1.0e-6;
}

#endif
