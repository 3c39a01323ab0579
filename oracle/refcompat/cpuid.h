/*
 * cpuid.h - stand-in for GCC's x86-only <cpuid.h> on other hosts
 * (TEST INFRASTRUCTURE ONLY).
 *
 * The reference includes <cpuid.h> in src/cpu/definitions.h:45 and
 * src/gpu/definitions.hpp:45 for one purpose: getCPUInfo (src/cpu/control.cpp,
 * src/gpu/control.cpp:177-203) reads the processor brand string through the
 * extended cpuid leaves and logs it. On an Arm host there is no cpuid
 * instruction; this macro reports no extended leaves, so the brand string is
 * empty and nothing else changes. oracle/ref_build.py and
 * oracle/ref_gpu_build.py put this directory on the include path only when
 * the host is not x86.
 */
#ifndef PFG_REFCOMPAT_CPUID_H
#define PFG_REFCOMPAT_CPUID_H

#define __cpuid(level, a, b, c, d) \
    do {                           \
        (void)(level);             \
        (a) = 0;                   \
        (b) = 0;                   \
        (c) = 0;                   \
        (d) = 0;                   \
    } while (0)

#endif
