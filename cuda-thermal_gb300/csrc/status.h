// status.h - error reporting for the C ABI: every entry point returns a
// ct_status and leaves a message for ct_last_error() on the calling thread.
#pragma once
#include <cstdarg>
#include <cstdio>

#include "cthermal.h"

namespace ct {

// Records a message for ct_last_error() and returns the status.
ct_status fail(ct_status s, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;

void clear_error();

}  // namespace ct
