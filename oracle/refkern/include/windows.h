// Stand-in for <windows.h>: the reference's stop-watch header needs only the
// high-resolution counter types.  The refkern build never calls them.
#pragma once
typedef union { long long QuadPart; } LARGE_INTEGER;
inline int QueryPerformanceFrequency(LARGE_INTEGER* p) { p->QuadPart = 1; return 1; }
inline int QueryPerformanceCounter(LARGE_INTEGER* p) { p->QuadPart = 0; return 1; }
