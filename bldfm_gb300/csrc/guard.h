// C-ABI entry points: C++ exceptions of the host side end at the C boundary.
#pragma once

#include "../../include/bldfm_gb300.h"

// Run an entry point's body; a C++ exception inside it (std::bad_alloc of a
// host allocation, a thread that cannot start) returns BLDFM_ERR_HOST
// instead of crossing the C boundary.
template <class F>
static inline int bldfm_guarded(F &&f)
{
    try {
        return f();
    } catch (...) {
        return BLDFM_ERR_HOST;
    }
}
