// guard.h -- no C++ exception crosses the C ABI.  Every exported function
// that returns a status runs its body through fpl_guard: a host allocation
// failure (std::bad_alloc from a container), a thread that cannot be started
// (std::system_error) or any other exception becomes FPL_ERR_HOST.
#pragma once
#include "fringe_gb300.h"

template <typename F>
inline int fpl_guard(F &&body) noexcept
{
    try {
        return body();
    } catch (...) {
        return FPL_ERR_HOST;
    }
}
