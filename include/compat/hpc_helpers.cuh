// hpc_helpers.cuh -- the reference's helper header name.  The reference's examples
// (example/mainatmos.cpp:19, example/mainbeam.cpp:20) and code written against them include
// it for its timer and utility macros; with include/compat/ on the include path they get this
// library's definitions of the same names and compile unchanged, with any C++14 compiler and
// no CUDA toolchain.
//
// What differs, on purpose: the library reports CUDA errors as status codes (the C++ facade
// turns them into std::runtime_error), so CUERR has nothing left to check and expands to
// nothing instead of printing and calling exit(1).
#pragma once

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>

// Wall-clock timers: TIMERSTART(label) ... TIMERSTOP(label) prints
// "# elapsed time (label): <seconds> s".  The *CPU variants are the same timers.
#define CP3_COMPAT_TIMER_BEGIN(label) \
    const auto cp3_compat_timer_##label = std::chrono::steady_clock::now();
#define CP3_COMPAT_TIMER_END(label)                                                         \
    std::cout << "# elapsed time (" << #label << "): "                                      \
              << std::chrono::duration<double>(std::chrono::steady_clock::now() -           \
                                               cp3_compat_timer_##label)                    \
                     .count()                                                               \
              << " s" << std::endl;
#define TIMERSTARTCPU(label) CP3_COMPAT_TIMER_BEGIN(label)
#define TIMERSTOPCPU(label) CP3_COMPAT_TIMER_END(label)
#define TIMERSTART(label) CP3_COMPAT_TIMER_BEGIN(label)
#define TIMERSTOP(label) CP3_COMPAT_TIMER_END(label)

#define CUERR

// ceil(x / y) for positive integers
#define SDIV(x, y) (((x) + (y) - 1) / (y))

// Function qualifiers: CUDA's when a CUDA compiler reads this header, empty otherwise.
#ifdef __CUDACC__
#define HOSTQUALIFIER __host__
#define DEVICEQUALIFIER __device__
#define HOSTDEVICEQUALIFIER __host__ __device__
#define KERNEL __global__
#define H2D (cudaMemcpyHostToDevice)
#define D2H (cudaMemcpyDeviceToHost)
#define H2H (cudaMemcpyHostToHost)
#define D2D (cudaMemcpyDeviceToDevice)
#else
#define HOSTQUALIFIER
#define DEVICEQUALIFIER
#define HOSTDEVICEQUALIFIER
#define KERNEL
#endif
#define UNROLLQUALIFIER
