// atag_internal.h — helpers shared between the library's host translation
// units (not part of the public C ABI).
#pragma once

#include "../../include/atag.h"

namespace atag {
// Records `msg` as this host thread's atag_last_error() and returns `s`.
atag_status set_error(atag_status s, const char* msg);
// Adds one to the launch counter reported by atag_launch_count().
void count_launch();
}  // namespace atag
