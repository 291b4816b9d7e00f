// Once-per-device guard for kernel attributes (cudaFuncSetAttribute applies
// to the current device's context): a call site keeps one flag word and
// sets its attributes when first_on_device() says the current device has not
// seen them yet.  Setting an attribute twice is harmless, so the unguarded
// read-modify-write of the word needs no lock.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

inline bool first_on_device(uint64_t &mask)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return true;
    const uint64_t bit = (uint64_t)1 << dev;
    if (mask & bit) return false;
    mask |= bit;
    return true;
}
